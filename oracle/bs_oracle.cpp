// bs_oracle.cpp -- TEST INFRASTRUCTURE ONLY: a CPU restatement of BioSpring's
// per-step force-and-integrate loop, used as the checker of the CUDA path.
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
// The product never links, loads or calls it.
//
// The restatement follows the reference's arithmetic operation by operation
// (same FP32/FP64 mix, same summation order, same neighbour-visit order) so
// that, on the machine where both are compiled, it reproduces the reference's
// forces and energies bit for bit; this is checked against the reference
// itself (oracle/ref.mk) by tests/test_oracle_pin.py through golden fixtures.
// A separate FP64 evaluator (bso_eval_fp64) gives the error statements.
//
// Reference functions restated here (paths inside the BioSpring project):
//   grid build / cell id / neighbour walk   src/nsearch.hpp:251-256, 277-319, 342-435
//   bounding box                            src/box.hpp:37-69
//   distance, norm                          src/measure.hpp:163-196, src/Vector3f.h:45-60
//   spring force + energy                   src/spn/Spring.cpp:20-34, energy/spring.hpp:17-29
//   steric (4 modes)                        src/spn/Particle.cpp:368-429, energy/steric.hpp:27-156
//   Coulomb                                 src/spn/Particle.cpp:191-253, energy/electrostatic.hpp:16-49
//   hydrophobic                             src/spn/Particle.cpp:269-330, energy/hydrophobic.hpp:20-39
//   IMPALA (flat membrane)                  src/spn/Particle.cpp:259-267, energy/imp.hpp:29-159,
//                                           src/forcefield/ForceField.cpp:62-88
//   viscosity, Euler step                   src/spn/Particle.cpp:80-84, 109-128
//   step order, deferred apply, energies    src/spn/SpringNetwork.cpp:63-268, 865-876
//   rigid bodies (single and multi-body)    src/rigidbody/RigidBody.cpp:57-162, 430-484, 567-635,
//                                           src/rigidbody/Quaternion.cpp:11-96
//
// Compile with -ffp-contract=off so that no multiply-add is fused.

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <unordered_set>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/biospring_gb300.h"

namespace
{

// ---- physical constants and unit conversions (src/forcefield/constants.hpp:36-118) ----
const double C_ELECTRONCHARGE_TO_COULOMB = 1.60217653E-19;
const double C_ANGSTROM_TO_METER = 1.0E-10;
const double C_METER_TO_ANGSTROM = 1.0E10;
const double C_DALTON_TO_KILOGRAM = 1.66054E-27;
const double C_KILOGRAM_TO_DALTON = 1.0 / C_DALTON_TO_KILOGRAM;
const double C_SECOND_TO_FEMTOSECOND = 1.0E15;
const double C_FEMTOSECOND_TO_SECOND = 1.0E-15;
const double C_KJOULE_TO_JOULE = 1.0E3;
const double C_JOULE_TO_KJOULE = 1.0E-3;
const double C_PI = 3.1415927;
const double C_VACUUMPERMITIVITY = 8.854187817E-12;
const double C_AVOGADRO = 6.02214169E23;
const double C_COULOMB_K = 1.0 / (4.0 * C_PI * C_VACUUMPERMITIVITY);
const double C_NEWTON_TO_DAFS2 = C_METER_TO_ANGSTROM * C_KILOGRAM_TO_DALTON * C_FEMTOSECOND_TO_SECOND * C_FEMTOSECOND_TO_SECOND;
const double C_BOLTZMANN_J_PER_K = 1.3806504E-23;
const double C_MIN_DIST_ELEC = 0.001;
const double C_MIN_DIST_VDW = 0.1;
const double C_KINETIC = (C_ANGSTROM_TO_METER * C_SECOND_TO_FEMTOSECOND) * (C_ANGSTROM_TO_METER * C_SECOND_TO_FEMTOSECOND) *
                         C_AVOGADRO * C_DALTON_TO_KILOGRAM * C_JOULE_TO_KJOULE;
const double C_SPRING_F = C_KJOULE_TO_JOULE / C_AVOGADRO * C_METER_TO_ANGSTROM * C_NEWTON_TO_DAFS2;
const double C_IMP_F = C_KJOULE_TO_JOULE / C_AVOGADRO * C_METER_TO_ANGSTROM * C_NEWTON_TO_DAFS2;
const double C_ELEC_F = C_NEWTON_TO_DAFS2 * (C_ELECTRONCHARGE_TO_COULOMB * C_ELECTRONCHARGE_TO_COULOMB) /
                        (C_VACUUMPERMITIVITY * C_ANGSTROM_TO_METER * C_ANGSTROM_TO_METER);
const float C_LINEAR_STIFFNESS = 1.0f;
const float C_ALIP = -0.018f;

// Overload resolution in the reference: the steric kernels are instantiated where the
// float overloads of <cmath> are visible, so pow(float, float) is the float function
// (and pow(a, b) / pow(c, d) is a float division); the hydrophobic and IMPALA kernels
// (compiled in ForceField.cpp) call the double exp. The pinning tests check this
// against the compiled reference bit for bit.
inline float rpow(float a, float b) { return ::powf(a, b); }
inline double rexp(double a) { return ::exp(a); }

struct V3
{
    float x, y, z;
};
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 mul(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 divs(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline V3 neg(V3 a) { return {-a.x, -a.y, -a.z}; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float dotf(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// measure::norm on a float vector (measure.hpp:188-196), returned as float (Vector3f::norm).
inline float norm3(V3 v)
{
    const double x = v.x, y = v.y, z = v.z;
    if (std::abs(x) < 1e-40 && std::abs(y) < 1e-40 && std::abs(z) < 1e-40)
        return 0.0f;
    return static_cast<float>(std::sqrt(x * x + y * y + z * z));
}
// Vector3f::normalize (Vector3f.h:45-60).
inline V3 normalize3(V3 v)
{
    const float n = norm3(v);
    if (n > 1.0E-40)
        return {v.x / n, v.y / n, v.z / n};
    return {0.0f, 0.0f, 0.0f};
}

// ---- force-field scalar kernels ---------------------------------------------------
struct FF
{
    int mode = BS_STERIC_LINEAR;
    float stericscale = 1, springscale = 1, impscale = 1, coulombscale = 1, hydroscale = 1, dielectric = 1;
    int dielectric_mode = BS_DIELECTRIC_CONSTANT;
    float imp_z0 = 15.75f, imp_alpha = 1.99f;
    // double membrane: offsets of the upper and lower membranes and their tube curvatures
    // (ForceField.h:23-25, 100-110); all zero for the flat membrane
    float memb_uo = 0.0f, memb_lo = 0.0f, memb_uc = 0.0f, memb_lc = 0.0f;
    bool flat() const { return memb_uo == 0.0f && memb_lo == 0.0f && memb_uc == 0.0f && memb_lc == 0.0f; }

    // One membrane of the double membrane (imp.hpp:33-62, 100-129): the tube radius (1e6 A when
    // flat), the curvature's sign, the z of the tube axis, the vector from that axis to the particle
    // and the particle's z in the membrane's frame. `off` is the membrane's signed offset (+upper,
    // -lower).
    struct Side
    {
        float radius;
        int sign;
        V3 rel;
        float depth;
    };
    static Side side(float x, float y, float z, float off, float curv)
    {
        Side d;
        d.radius = curv == 0.0f ? 1000000.0f : std::abs(1 / curv);
        d.sign = (curv > 0.0f) - (curv < 0.0f);
        const V3 centre = {0.0f, y, off - d.sign * d.radius};
        d.rel = sub(V3{x, y, z}, centre);
        if (d.sign == 0)
            d.depth = z;
        else if (z > centre.z)
            d.depth = d.sign * norm3(d.rel) + off - d.radius;
        else
            d.depth = -d.sign * norm3(d.rel) + off - d.radius;
        return d;
    }
    // imp.hpp:29-77 with the double-membrane parameters set
    float imp_energy_double(float x, float y, float z, float surface, float transfer) const
    {
        const Side u = side(x, y, z, memb_uo, memb_uc), l = side(x, y, z, -memb_lo, memb_lc);
        const double cu = 0.5 - 1.0 / (1.0 + rexp(imp_alpha * (std::abs(u.depth - memb_uo) - imp_z0)));
        const double cl = 0.5 - 1.0 / (1.0 + rexp(imp_alpha * (std::abs(l.depth + memb_lo) - imp_z0)));
        const double hu = -surface * transfer * cu, hl = -surface * transfer * cl;
        const double lu = C_ALIP * surface * cu, ll = C_ALIP * surface * cl;
        return impscale * static_cast<float>(hu + lu + hl + ll);
    }
    // imp.hpp:88-159 with the double-membrane parameters set, ForceField.cpp:80-85
    V3 imp_force_double(float x, float y, float z, float surface, float transfer) const
    {
        const Side u = side(x, y, z, memb_uo, memb_uc), l = side(x, y, z, -memb_lo, memb_lc);
        auto expo = [&](float zz, float off) { return rexp(imp_alpha * (std::abs(zz + off) - imp_z0)); };
        double du = (imp_alpha * (u.depth - memb_uo) * expo(u.depth, -memb_uo)) /
                    (std::pow(expo(u.depth, -memb_uo) + 1, 2.0) * std::abs(u.depth - memb_uo));
        double dl = (imp_alpha * (l.depth + memb_lo) * expo(l.depth, memb_lo)) /
                    (std::pow(expo(l.depth, memb_lo) + 1, 2.0) * std::abs(l.depth + memb_lo));
        if (std::isnan(du) || !std::isfinite(du))
            du = 0.0;
        if (std::isnan(dl) || !std::isfinite(dl))
            dl = 0.0;
        const V3 dir_u = normalize3(u.sign == 0 ? V3{0.0f, 0.0f, 1.0f} : u.rel);
        const V3 dir_l = normalize3(l.sign == 0 ? V3{0.0f, 0.0f, 1.0f} : l.rel);
        const double hu = -surface * transfer * du, hl = -surface * transfer * dl;
        const double lu = C_ALIP * surface * du, ll = C_ALIP * surface * dl;
        const V3 fu = mul(dir_u, static_cast<float>((hu + lu) * C_IMP_F));
        const V3 fl = mul(dir_l, static_cast<float>((hl + ll) * C_IMP_F));
        return mul(neg(add(fu, fl)), impscale);
    }

    // spring.hpp:17-29 wrapped by ForceField.cpp:39-47
    float spring_energy(float d, float k, float r0) const
    {
        float dv = d - r0;
        return springscale * static_cast<float>(0.5 * k * dv * dv);
    }
    float spring_force(float d, float k, float r0) const
    {
        float fm = k * (d - r0);
        fm = static_cast<float>(fm * C_SPRING_F);
        return springscale * fm;
    }

    // steric.hpp:27-156 wrapped by the ForceField subclasses (radius_i = neighbour, radius_j = self)
    float steric_energy(float ri, float rj, float ei, float ej, float d) const
    {
        float e = 0.0f;
        if (mode == BS_STERIC_LINEAR)
        {
            float eq = ri + rj;
            float dv = d - eq;
            e = dv > 0 ? 0.0f : static_cast<float>(0.5 * C_LINEAR_STIFFNESS * dv * dv);
        }
        else
        {
            if (d < C_MIN_DIST_VDW)
                return stericscale * 0.0f;
            if (mode == BS_STERIC_LJ_12_6_AMBER)
            {
                float eij = std::sqrt(ei * ej), rij = std::sqrt(ri * rj);
                float rep = static_cast<float>(eij * rpow(rij / d, 12.0f));
                float att = static_cast<float>(-eij * 2.0 * rpow(rij / d, 6.0f));
                e = rep + att;
            }
            else if (mode == BS_STERIC_LJ_8_6_LEWITT)
            {
                float eij = std::sqrt(ei * ej), rij = std::sqrt(ri * rj);
                float rep = static_cast<float>(eij * 3.0 * rpow(rij / d, 8.0f));
                float att = static_cast<float>(-eij * 4.0 * rpow(rij / d, 6.0f));
                e = rep + att;
            }
            else
            {
                float eij = ei * ej, rij = ri * rj;
                float rep = static_cast<float>(eij * rpow(rij / d, 8.0f));
                float att = static_cast<float>(-eij * rpow(rij / d, 6.0f));
                e = rep + att;
            }
        }
        return stericscale * e;
    }
    float steric_force(float ri, float rj, float ei, float ej, float d) const
    {
        float fm = 0.0f;
        if (mode == BS_STERIC_LINEAR)
        {
            float eq = ri + rj;
            float dv = d - eq;
            if (dv > 0)
                fm = 0.0f;
            else
            {
                float m = -C_LINEAR_STIFFNESS * std::fabs(dv);
                fm = static_cast<float>(m * C_SPRING_F);
            }
        }
        else
        {
            if (d < C_MIN_DIST_VDW)
                return stericscale * 0.0f;
            float rep, att;
            if (mode == BS_STERIC_LJ_12_6_AMBER)
            {
                float eij = std::sqrt(ei * ej), rij = std::sqrt(ri * rj);
                rep = static_cast<float>(-eij * 12.0 * (rpow(rij, 12.0f) / rpow(d, 13.0f)));
                att = static_cast<float>(eij * 2.0 * 6.0 * (rpow(rij, 6.0f) / rpow(d, 7.0f)));
            }
            else if (mode == BS_STERIC_LJ_8_6_LEWITT)
            {
                float eij = std::sqrt(ei * ej), rij = std::sqrt(ri * rj);
                rep = static_cast<float>(-eij * 3.0 * 8.0 * (rpow(rij, 8.0f) / rpow(d, 9.0f)));
                att = static_cast<float>(eij * 4.0 * 6.0 * (rpow(rij, 6.0f) / rpow(d, 7.0f)));
            }
            else
            {
                float eij = ei * ej, rij = ri * rj;
                rep = static_cast<float>(-eij * 8.0 * (rpow(rij, 8.0f) / rpow(d, 9.0f)));
                att = static_cast<float>(eij * 6.0 * (rpow(rij, 6.0f) / rpow(d, 7.0f)));
            }
            float m = rep + att;
            fm = static_cast<float>(m * C_SPRING_F);
        }
        return stericscale * fm;
    }

    // electrostatic.hpp:16-49 wrapped by ForceField.cpp:27-35. With the distance-dependent
    // dielectric (no reference counterpart) eps = dielectric * d and the force is -dE/dd.
    float elec_energy(float q1, float q2, float d) const
    {
        if (d < C_MIN_DIST_ELEC)
            return coulombscale * 0.0f;
        double k = C_COULOMB_K;
        double a = q1 * C_ELECTRONCHARGE_TO_COULOMB;
        double b = q2 * C_ELECTRONCHARGE_TO_COULOMB;
        float eps = dielectric_mode == BS_DIELECTRIC_DISTANCE ? dielectric * d : dielectric;
        float dm = static_cast<float>(d * C_ANGSTROM_TO_METER);
        double e = k * (a * b) / (eps * dm);
        e = e * C_AVOGADRO;
        e = e * 1.0E-3;
        return coulombscale * static_cast<float>(e);
    }
    float elec_force(float q1, float q2, float d) const
    {
        if (d < C_MIN_DIST_ELEC)
            return coulombscale * 0.0f;
        float fm;
        if (dielectric_mode == BS_DIELECTRIC_DISTANCE)
        {
            float eps = dielectric * d;
            fm = static_cast<float>(-2.0f * (q1 * q2) / (4.0 * C_PI * eps * d * d));
        }
        else
            fm = static_cast<float>(-(q1 * q2) / (4.0 * C_PI * dielectric * d * d));
        fm = static_cast<float>(fm * C_ELEC_F);
        return coulombscale * fm;
    }

    // hydrophobic.hpp:20-39 wrapped by ForceField.cpp:73-80
    float hydro_energy(float h1, float h2, float d) const
    {
        double e = -(h1 * h2) * rexp(-d);
        e = e * C_AVOGADRO;
        e = e * 1.0E-3;
        return hydroscale * static_cast<float>(e);
    }
    float hydro_force(float h1, float h2, float d) const
    {
        float fm = static_cast<float>((h1 * h2) * rexp(-d));
        fm = static_cast<float>(fm * C_SPRING_F);
        return hydroscale * fm;
    }

    // imp.hpp:29-77 (flat membrane: offsets and curvatures are 0 in the reference run)
    float imp_energy(float z, float surface, float transfer) const
    {
        const float alpha = imp_alpha, z0 = imp_z0;
        double cz = 0.5 - 1.0 / (1.0 + rexp(alpha * (std::abs(z - 0.0f) - z0)));
        double hydro = -surface * transfer * cz;
        double lipid = C_ALIP * surface * cz;
        return impscale * static_cast<float>(hydro + lipid);
    }
    // imp.hpp:88-159 and ForceField.cpp:84-88 (the vector is negated, then scaled)
    V3 imp_force(float z, float surface, float transfer) const
    {
        const float alpha = imp_alpha, z0 = imp_z0;
        auto expo = [&](float zz, float off) { return rexp(alpha * (std::abs(zz + off) - z0)); };
        double dcz = (alpha * (z - 0.0f) * expo(z, -0.0f)) / (std::pow(expo(z, -0.0f) + 1, 2.0) * std::abs(z - 0.0f));
        if (std::isnan(dcz) || !std::isfinite(dcz))
            dcz = 0.0;
        double hydro = -surface * transfer * dcz;
        double lipid = C_ALIP * surface * dcz;
        const float s = static_cast<float>((hydro + lipid) * C_IMP_F);
        V3 f = {0.0f * s, 0.0f * s, 1.0f * s};
        f = neg(f);
        return mul(f, impscale);
    }
};

// ---- reference cell grid (nsearch.hpp:155-436) ---------------------------------
struct Grid
{
    bool active = false;
    float cutoff = 0.0f, skin = 0.0f;
    std::vector<int64_t> included; // empty = every particle
    double minx = 0, miny = 0, minz = 0;
    size_t nx = 1, ny = 1, nz = 1;
    std::vector<int64_t> start, items; // counting-sorted cell contents, ascending index inside a cell
    std::vector<std::array<double, 3>> refpos;

    float radius() const { return cutoff + skin; }

    size_t cell_of(double px, double py, double pz) const
    {
        const float r = radius();
        size_t cy = static_cast<size_t>((py - miny) / r);
        size_t cz = static_cast<size_t>((pz - minz) / r);
        size_t cx = static_cast<size_t>((px - minx) / r);
        cx = std::min(cx, nx - 1);
        cy = std::min(cy, ny - 1);
        cz = std::min(cz, nz - 1);
        return cx + cy * nx + cz * nx * ny;
    }

    void build(const std::vector<float> & x, const std::vector<float> & y, const std::vector<float> & z)
    {
        const size_t n = x.size();
        double mnx = x[0], mny = y[0], mnz = z[0], mxx = x[0], mxy = y[0], mxz = z[0];
        for (size_t i = 1; i < n; ++i)
        {
            double a = x[i], b = y[i], c = z[i];
            if (a < mnx) mnx = a;
            if (b < mny) mny = b;
            if (c < mnz) mnz = c;
            if (a > mxx) mxx = a;
            if (b > mxy) mxy = b;
            if (c > mxz) mxz = c;
        }
        minx = mnx;
        miny = mny;
        minz = mnz;
        const float r = radius();
        nx = size_t(std::ceil((mxx - mnx) / r) + 1);
        ny = size_t(std::ceil((mxy - mny) / r) + 1);
        nz = size_t(std::ceil((mxz - mnz) / r) + 1);
        const size_t nc = nx * ny * nz;
        std::vector<size_t> cellid;
        std::vector<int64_t> members;
        if (included.empty())
        {
            members.resize(n);
            for (size_t i = 0; i < n; ++i)
                members[i] = static_cast<int64_t>(i);
        }
        else
            members = included;
        cellid.resize(members.size());
        start.assign(nc + 1, 0);
        for (size_t m = 0; m < members.size(); ++m)
        {
            const int64_t i = members[m];
            cellid[m] = cell_of(x[i], y[i], z[i]);
            start[cellid[m] + 1]++;
        }
        for (size_t c = 0; c < nc; ++c)
            start[c + 1] += start[c];
        items.assign(members.size(), 0);
        std::vector<int64_t> fill(start.begin(), start.end() - 1);
        for (size_t m = 0; m < members.size(); ++m)
            items[fill[cellid[m]]++] = members[m];
        if (skin > 0.0f)
        {
            refpos.assign(n, {0, 0, 0});
            for (int64_t i : members)
                refpos[i] = {static_cast<double>(x[i]), static_cast<double>(y[i]), static_cast<double>(z[i])};
        }
    }

    // NeighborSearch::_exceeds_skin (nsearch.hpp:405-435)
    bool exceeds_skin(const std::vector<float> & x, const std::vector<float> & y, const std::vector<float> & z) const
    {
        if (skin <= 0.0f)
            return true;
        auto drift = [&](int64_t i) {
            const double dx = x[i] - refpos[i][0], dy = y[i] - refpos[i][1], dz = z[i] - refpos[i][2];
            return std::sqrt(dx * dx + dy * dy + dz * dz) > static_cast<double>(skin);
        };
        if (included.empty())
        {
            for (size_t i = 0; i < x.size(); ++i)
                if (drift(static_cast<int64_t>(i)))
                    return true;
        }
        else
            for (int64_t i : included)
                if (drift(i))
                    return true;
        return false;
    }

    // for_each_neighbor (nsearch.hpp:214-234, 295-319): 27 cells in dx, dy, dz order,
    // candidates filtered by the double distance < cutoff, self excluded.
    template <typename CB>
    void for_each_neighbor(int64_t self, const std::vector<float> & x, const std::vector<float> & y,
                           const std::vector<float> & z, CB && cb) const
    {
        const double px = x[self], py = y[self], pz = z[self];
        const size_t cell = cell_of(px, py, pz);
        const int cx = static_cast<int>(cell % nx), cy = static_cast<int>((cell / nx) % ny),
                  cz = static_cast<int>(cell / (nx * ny));
        for (int dx = -1; dx <= 1; dx++)
            for (int dy = -1; dy <= 1; dy++)
                for (int dz = -1; dz <= 1; dz++)
                {
                    const int ax = cx + dx, ay = cy + dy, az = cz + dz;
                    if (ax < 0 || ax >= static_cast<int>(nx) || ay < 0 || ay >= static_cast<int>(ny) || az < 0 ||
                        az >= static_cast<int>(nz))
                        continue;
                    const size_t c = static_cast<size_t>(ax) + static_cast<size_t>(ay) * nx +
                                     static_cast<size_t>(az) * nx * ny;
                    for (int64_t k = start[c]; k < start[c + 1]; ++k)
                    {
                        const int64_t j = items[k];
                        if (j == self)
                            continue;
                        const double ddx = px - static_cast<double>(x[j]);
                        const double ddy = py - static_cast<double>(y[j]);
                        const double ddz = pz - static_cast<double>(z[j]);
                        if (std::sqrt(ddx * ddx + ddy * ddy + ddz * ddz) < cutoff)
                            cb(j);
                    }
                }
    }
};

struct Deferred
{
    int64_t target;
    V3 f;
    float e;
};

struct Body
{
    std::vector<int64_t> ids;
    double mass = 0;
    V3 pos{0, 0, 0}, v{0, 0, 0}, a{0, 0, 0}, L{0, 0, 0}, omega{0, 0, 0}, force{0, 0, 0}, torque{0, 0, 0};
    float q[4] = {0, 0, 0, 1}; // x, y, z, w
    std::vector<V3> p0;
    double ibodyinv = 0; // inverse of the diagonal sphere inertia (RigidBody.cpp:105-108)
};

// Quaternion algebra of src/rigidbody/Quaternion.cpp (x, y, z, w in float).
struct Q
{
    float x, y, z, w;
};
inline Q qmul(Q a, Q b)
{
    V3 v2{b.x, b.y, b.z}, v1{a.x, a.y, a.z};
    V3 ax1 = mul(v2, a.w), ax2 = mul(v1, b.w), ax3 = cross(v1, v2);
    V3 ax = add(add(ax1, ax2), ax3);
    return {ax.x, ax.y, ax.z, a.w * b.w - dotf(v1, v2)};
}
inline void qnormalize(Q & q)
{
    float m = std::sqrt(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
    if (m > 0.005)
    {
        q.x /= m;
        q.y /= m;
        q.z /= m;
        q.w /= m;
    }
}
inline Q qinverse(Q q)
{
    float a = std::sqrt(q.w * q.w + q.x * q.x + q.y * q.y + q.z * q.z);
    a *= a;
    a = 1 / a;
    Q c{-q.x, -q.y, -q.z, q.w};
    float s = c.w * a;
    V3 im = mul(V3{c.x, c.y, c.z}, a);
    return {im.x, im.y, im.z, s};
}

// A field grid (PotentialGrid, src/grid/PotentialGrid.hpp): scalar and force vector per cell,
// OpenDX order, over the box [lo, hi] (GridCoordinatesSystem.hpp:154-218).
struct Field
{
    bool on = false;
    int n[3] = {0, 0, 0};
    double o[3] = {0, 0, 0}, h[3] = {1, 1, 1}, hi[3] = {0, 0, 0};
    std::vector<float> sc, gx, gy, gz;

    // PotentialGrid::compute_gradient (PotentialGrid.cpp:20-59)
    void set(const int32_t shape[3], const double origin[3], const double spacing[3], const float * scalar)
    {
        for (int a = 0; a < 3; ++a)
        {
            n[a] = shape[a];
            o[a] = origin[a];
            h[a] = spacing[a];
            hi[a] = origin[a] + static_cast<double>(static_cast<size_t>(shape[a])) * spacing[a];
        }
        const size_t total = static_cast<size_t>(n[0]) * n[1] * n[2];
        sc.assign(scalar, scalar + total);
        gx.assign(total, 0.0f);
        gy.assign(total, 0.0f);
        gz.assign(total, 0.0f);
        const float scale = static_cast<float>(C_BOLTZMANN_J_PER_K * C_METER_TO_ANGSTROM * C_NEWTON_TO_DAFS2);
        const float dx = static_cast<float>(h[0]), dy = static_cast<float>(h[1]), dz = static_cast<float>(h[2]);
        auto id = [&](size_t i, size_t j, size_t k) { return (i * n[1] + j) * n[2] + k; };
        auto grad = [](float cur, float prev, float next, float cs) -> float {
            return ((cur - prev) + (next - cur)) / (cs * 2.0);
        };
        for (size_t i = 0; i < static_cast<size_t>(n[0]); ++i)
            for (size_t j = 0; j < static_cast<size_t>(n[1]); ++j)
                for (size_t k = 0; k < static_cast<size_t>(n[2]); ++k)
                {
                    const size_t c = id(i, j, k);
                    V3 g{0.0f, 0.0f, 0.0f};
                    if (i > 0 && i < static_cast<size_t>(n[0]) - 1)
                        g.x = grad(sc[c], sc[id(i - 1, j, k)], sc[id(i + 1, j, k)], dx);
                    if (j > 0 && j < static_cast<size_t>(n[1]) - 1)
                        g.y = grad(sc[c], sc[id(i, j - 1, k)], sc[id(i, j + 1, k)], dy);
                    if (k > 0 && k < static_cast<size_t>(n[2]) - 1)
                        g.z = grad(sc[c], sc[id(i, j, k - 1)], sc[id(i, j, k + 1)], dz);
                    g = mul(g, -scale);
                    gx[c] = g.x;
                    gy[c] = g.y;
                    gz[c] = g.z;
                }
    }

    // the cell holding (x, y, z), or -1 outside the box (is_out_of_grid, then cell_coordinates:
    // GridCoordinatesSystem.hpp:85-94, 206-218)
    int64_t cell(float x, float y, float z) const
    {
        const double p[3] = {x, y, z};
        int c[3];
        for (int a = 0; a < 3; ++a)
        {
            if (p[a] < o[a] || p[a] > hi[a] - 1e-6)
                return -1;
            c[a] = static_cast<int>((p[a] - o[a]) / h[a]);
        }
        return (static_cast<int64_t>(c[0]) * n[1] + c[1]) * n[2] + c[2];
    }
};

struct Sim
{
    bs_config cfg{};
    Field field[2]; // potential (electrostatic field), density
    std::vector<float> burying;
    FF ff;
    int64_t n = 0;
    std::vector<float> x, y, z, vx, vy, vz, fx, fy, fz, mass, charge, radius, eps, hydro, sasa, transfer;
    std::vector<float> pe_elec, pe_steric, pe_imp, pe_hydro, pe_kin;
    std::vector<uint8_t> is_static, charged, hydrophobic, rigid;
    std::vector<int32_t> body_of;
    std::vector<int64_t> dynamic;
    // springs in insertion order (deduplicated), and the bonded-partner sets
    std::vector<int64_t> s_i, s_j;
    std::vector<float> s_r0, s_k, s_energy;
    std::vector<int64_t> dyn_springs;
    std::vector<std::unordered_set<int64_t>> bonded;
    Grid grid[3];
    float energies[BS_NUM_ENERGIES] = {0, 0, 0, 0, 0, 0};
    // probe particle (SpringNetwork.cpp:749-766): not in the particle lists or the grids
    struct Probe
    {
        V3 pos{1, 1, 1}, vel{0, 0, 0}, force{0, 0, 0};
        float mass = 1, radius = 1, eps = 1, charge = 0;
    } probe;
    bool probe_on = false;
    std::vector<Body> bodies;
    bool rigid_on = false;

    V3 pos(int64_t i) const { return {x[i], y[i], z[i]}; }
    V3 vel(int64_t i) const { return {vx[i], vy[i], vz[i]}; }
    void add_force(int64_t i, V3 f)
    {
        fx[i] = fx[i] + f.x;
        fy[i] = fy[i] + f.y;
        fz[i] = fz[i] + f.z;
    }
    void reset_force(int64_t i)
    {
        fx[i] = fy[i] = fz[i] = 0.0f;
        pe_elec[i] = pe_steric[i] = pe_kin[i] = pe_imp[i] = pe_hydro[i] = 0.0f;
    }

    void setup_grids()
    {
        for (auto & g : grid)
            g.active = false;
        if (cfg.steric_enable)
        {
            grid[0].active = true;
            grid[0].cutoff = static_cast<float>(cfg.steric_cutoff);
            grid[0].skin = static_cast<float>(cfg.neighborskin);
            grid[0].included.clear();
            grid[0].build(x, y, z);
        }
        if (cfg.coulomb_enable)
        {
            grid[1].included.clear();
            for (int64_t i = 0; i < n; ++i)
                if (charged[i])
                    grid[1].included.push_back(i);
            if (!grid[1].included.empty())
            {
                grid[1].active = true;
                grid[1].cutoff = static_cast<float>(cfg.coulomb_cutoff);
                grid[1].skin = static_cast<float>(cfg.neighborskin);
                grid[1].build(x, y, z);
            }
        }
        if (cfg.hydrophobicity_enable)
        {
            grid[2].included.clear();
            for (int64_t i = 0; i < n; ++i)
                if (hydrophobic[i])
                    grid[2].included.push_back(i);
            if (!grid[2].included.empty())
            {
                grid[2].active = true;
                grid[2].cutoff = static_cast<float>(cfg.hydrophobicity_cutoff);
                grid[2].skin = static_cast<float>(cfg.neighborskin);
                grid[2].build(x, y, z);
            }
        }
    }

    void update_grids()
    {
        for (auto & g : grid)
            if (g.active && g.exceeds_skin(x, y, z))
                g.build(x, y, z);
    }

    // SpringNetwork::computeSpringForces (SpringNetwork.cpp:63-90)
    void compute_spring_forces()
    {
        float springenergy = 0.0f;
        std::vector<V3> scratch(dyn_springs.size());
#pragma omp parallel for schedule(static)
        for (int64_t t = 0; t < static_cast<int64_t>(dyn_springs.size()); ++t)
        {
            const int64_t s = dyn_springs[t];
            const int64_t a = s_i[s], b = s_j[s];
            s_energy[s] = 0.0f;
            if ((rigid[a] && rigid[b]) || (is_static[a] && is_static[b]))
            {
                scratch[t] = {0, 0, 0};
                continue;
            }
            const V3 disp = sub(pos(b), pos(a));
            const float len = norm3(disp);
            s_energy[s] = ff.spring_energy(len, s_k[s], s_r0[s]);
            const V3 dir = normalize3(disp);
            scratch[t] = mul(dir, ff.spring_force(len, s_k[s], s_r0[s]));
        }
        for (size_t t = 0; t < dyn_springs.size(); ++t)
        {
            const int64_t s = dyn_springs[t];
            add_force(s_i[s], scratch[t]);
            add_force(s_j[s], neg(scratch[t]));
            springenergy += s_energy[s];
        }
        energies[BS_ENERGY_SPRING] = springenergy;
    }

    // One nonbonded term for particle i (Particle.cpp:191-253, 269-330, 368-429).
    template <int TERM> void pair_term(int64_t i, std::vector<Deferred> & deferred)
    {
        const Grid & g = grid[TERM];
        const float cutoff = g.cutoff;
        g.for_each_neighbor(i, x, y, z, [&](int64_t j) {
            if (!is_static[j] && j < i)
                return;
            if (cfg.spring_enable && bonded[i].count(j))
                return;
            if (TERM == BS_TERM_STERIC && j == i)
                return;
            V3 f = sub(pos(j), pos(i));
            const float d = norm3(f);
            if (TERM == BS_TERM_STERIC)
            {
                if (!(d < cutoff))
                    return;
            }
            else if (!(d < cutoff && d != 0.0))
                return;
            float pe;
            float m;
            if (TERM == BS_TERM_STERIC)
            {
                pe = ff.steric_energy(radius[j], radius[i], eps[j], eps[i], d);
                f = normalize3(f);
                m = ff.steric_force(radius[j], radius[i], eps[j], eps[i], d);
            }
            else if (TERM == BS_TERM_COULOMB)
            {
                pe = ff.elec_energy(charge[j], charge[i], d);
                f = normalize3(f);
                m = ff.elec_force(charge[j], charge[i], d);
            }
            else
            {
                pe = ff.hydro_energy(hydro[j], hydro[i], d);
                f = normalize3(f);
                m = ff.hydro_force(hydro[j], hydro[i], d);
            }
            f = mul(f, m);
            add_force(i, f);
            float & own = TERM == BS_TERM_STERIC ? pe_steric[i] : (TERM == BS_TERM_COULOMB ? pe_elec[i] : pe_hydro[i]);
            if (!is_static[j])
            {
                const float half = TERM == BS_TERM_COULOMB ? 0.5f * pe : pe / 2.0f;
                own += half;
                deferred.push_back({j, neg(f), half});
            }
            else
                own += pe;
        });
    }

    // SpringNetwork::computeParticleForces (SpringNetwork.cpp:93-198)
    void compute_particle_forces()
    {
        float e_elec = 0.0f, e_steric = 0.0f, e_imp = 0.0f, e_hydro = 0.0f;
        const size_t nd = dynamic.size();
        std::vector<std::vector<Deferred>> d_steric(nd), d_elec(nd), d_hydro(nd);
        const float visc = static_cast<float>(cfg.viscosity_value);
#pragma omp parallel for schedule(static)
        for (int64_t t = 0; t < static_cast<int64_t>(nd); ++t)
        {
            const int64_t i = dynamic[t];
            if (cfg.coulomb_enable && charged[i] && grid[1].active)
                pair_term<BS_TERM_COULOMB>(i, d_elec[t]);
            if (cfg.coulomb_enable && field[0].on)
            {
                // Particle::addElectrostaticFieldForce (Particle.cpp:161-189)
                const int64_t c = field[0].cell(x[i], y[i], z[i]);
                if (c >= 0)
                {
                    const float gs = static_cast<float>(cfg.potentialgrid_scale);
                    const V3 v{field[0].gx[c], field[0].gy[c], field[0].gz[c]};
                    add_force(i, mul(mul(v, charge[i]), gs));
                    // electrostatic_field_energy (electrostatic_field.hpp:16-23) times the scale
                    float en = field[0].sc[c] * charge[i];
                    en = en * C_BOLTZMANN_J_PER_K;
                    en = en * C_JOULE_TO_KJOULE;
                    en = en * C_AVOGADRO;
                    pe_elec[i] += gs * en;
                }
            }
            if (field[1].on)
            {
                // Particle::addDensityFieldForce (Particle.cpp:136-159)
                const int64_t c = field[1].cell(x[i], y[i], z[i]);
                if (c >= 0)
                {
                    const float gs = static_cast<float>(cfg.densitygrid_scale);
                    const V3 v{field[1].gx[c], field[1].gy[c], field[1].gz[c]};
                    add_force(i, mul(mul(v, burying.empty() ? 1.0f : burying[i]), gs));
                }
            }
            if (cfg.steric_enable)
                pair_term<BS_TERM_STERIC>(i, d_steric[t]);
            if (cfg.viscosity_enable)
            {
                const V3 vs = mul(vel(i), visc);
                fx[i] = fx[i] - vs.x;
                fy[i] = fy[i] - vs.y;
                fz[i] = fz[i] - vs.z;
            }
            if (cfg.impala_enable)
            {
                if (ff.flat())
                {
                    pe_imp[i] = ff.imp_energy(z[i], sasa[i], transfer[i]);
                    add_force(i, ff.imp_force(z[i], sasa[i], transfer[i]));
                }
                else
                {
                    pe_imp[i] = ff.imp_energy_double(x[i], y[i], z[i], sasa[i], transfer[i]);
                    add_force(i, ff.imp_force_double(x[i], y[i], z[i], sasa[i], transfer[i]));
                }
            }
            if (cfg.hydrophobicity_enable && hydrophobic[i] && grid[2].active)
                pair_term<BS_TERM_HYDROPHOBIC>(i, d_hydro[t]);
        }
        auto apply = [&](const std::vector<std::vector<Deferred>> & scratch, float & e) {
            for (const auto & bucket : scratch)
                for (const auto & c : bucket)
                {
                    add_force(c.target, c.f);
                    e += c.e;
                }
        };
        apply(d_steric, e_steric);
        apply(d_elec, e_elec);
        apply(d_hydro, e_hydro);
        for (int64_t i : dynamic)
        {
            e_elec += pe_elec[i];
            e_steric += pe_steric[i];
            e_imp += pe_imp[i];
            e_hydro += pe_hydro[i];
        }
        float probe_ke = 0.0f;
        if (probe_on)
        {
            // SpringNetwork.cpp:156-182 and Particle::addStericProbeForce /
            // addElectrostaticProbeForce (Particle.cpp:434-465): every dynamic particle against the
            // probe, no cutoff, full pair energy to the totals; then the probe alone moves.
            probe.force = {0, 0, 0};
            for (int64_t i : dynamic)
            {
                if (cfg.probe_steric)
                {
                    V3 f = sub(probe.pos, pos(i));
                    const float d = norm3(f);
                    const float pe = ff.steric_energy(probe.radius, radius[i], probe.eps, eps[i], d);
                    pe_steric[i] += pe * 0.5f;
                    f = normalize3(f);
                    f = mul(f, ff.steric_force(probe.radius, radius[i], probe.eps, eps[i], d));
                    add_force(i, f);
                    probe.force = add(probe.force, neg(f));
                    e_steric += pe;
                }
                if (cfg.probe_electrostatic)
                {
                    V3 f = sub(probe.pos, pos(i));
                    const float d = norm3(f);
                    const float pe = ff.elec_energy(probe.charge, charge[i], d);
                    pe_elec[i] += pe * 0.5f;
                    f = normalize3(f);
                    f = mul(f, ff.elec_force(probe.charge, charge[i], d));
                    add_force(i, f);
                    probe.force = add(probe.force, neg(f));
                    e_elec += pe;
                }
            }
            if (cfg.viscosity_enable)
                probe.force = sub(probe.force, mul(probe.vel, visc));
            // Particle::IntegrateEuler (Particle.cpp:109-128)
            const float dt = static_cast<float>(cfg.timestep);
            if (probe.mass > 0.0f)
                probe.vel = add(probe.vel, mul(divs(probe.force, probe.mass), dt));
            const float vit = norm3(probe.vel);
            probe_ke = static_cast<float>(0.5f * probe.mass * (vit * vit) * C_KINETIC);
            probe.pos = add(probe.pos, mul(probe.vel, dt));
        }
        if (rigid_on)
            for (int64_t i : dynamic)
                if (rigid[i])
                {
                    // RigidBody::computeParticleForceAndTorque (RigidBody.cpp:567-580)
                    Body & b = bodies[body_of[i]];
                    const V3 f{fx[i], fy[i], fz[i]};
                    V3 tq{0, 0, 0};
                    tq = add(tq, cross(sub(pos(i), b.pos), f));
                    b.force = add(b.force, f);
                    b.torque = add(b.torque, tq);
                }
        energies[BS_ENERGY_KINETIC] += probe_ke; // before the particles' kinetic energy
        energies[BS_ENERGY_ELECTROSTATIC] = e_elec;
        energies[BS_ENERGY_STERIC] = e_steric;
        energies[BS_ENERGY_IMP] = e_imp;
        energies[BS_ENERGY_HYDROPHOBIC] = e_hydro;
    }

    // RigidBody::solve, dynamics branch (RigidBody.cpp:455-483)
    void solve_bodies()
    {
        const double dt = static_cast<float>(cfg.timestep);
        for (Body & b : bodies)
        {
            b.a = divs(b.force, static_cast<float>(b.mass));
            b.v = add(b.v, mul(b.a, static_cast<float>(dt)));
            const V3 t1 = mul(b.v, static_cast<float>(dt));
            V3 t2 = mul(b.a, 0.5f);
            t2 = mul(t2, static_cast<float>(dt));
            t2 = mul(t2, static_cast<float>(dt));
            b.pos = add(b.pos, add(t1, t2));
            b.L = add(b.L, mul(b.torque, static_cast<float>(dt)));
            const double ox = b.ibodyinv * b.L.x + 0.0 * b.L.y + 0.0 * b.L.z;
            const double oy = 0.0 * b.L.x + b.ibodyinv * b.L.y + 0.0 * b.L.z;
            const double oz = 0.0 * b.L.x + 0.0 * b.L.y + b.ibodyinv * b.L.z;
            b.omega = {static_cast<float>(ox), static_cast<float>(oy), static_cast<float>(oz)};
            const float angle = static_cast<float>(norm3(b.omega) * dt);
            const float sa = static_cast<float>(std::sin(angle / 2.0));
            const float ca = static_cast<float>(std::cos(angle / 2.0));
            Q dq{b.omega.x * sa, b.omega.y * sa, b.omega.z * sa, ca};
            qnormalize(dq);
            Q q{b.q[0], b.q[1], b.q[2], b.q[3]};
            q = qmul(dq, q);
            qnormalize(q);
            b.q[0] = q.x;
            b.q[1] = q.y;
            b.q[2] = q.z;
            b.q[3] = q.w;
            b.force = {0, 0, 0};
            b.torque = {0, 0, 0};
        }
    }

    // SpringNetwork::updateParticlePositions (SpringNetwork.cpp:202-241). Returns false on a
    // non-finite position.
    bool update_positions()
    {
        const float dt = static_cast<float>(cfg.timestep);
        float ke = 0.0f;
        bool finite = true;
        for (size_t t = 0; t < dynamic.size(); ++t)
        {
            const int64_t i = dynamic[t];
            if (rigid_on && rigid[i])
            {
                // RigidBody::integrateParticleVelocity (RigidBody.cpp:600-635), with the
                // particle's index inside its own body.
                const Body & b = bodies[body_of[i]];
                const V3 prev = pos(i);
                const size_t local = static_cast<size_t>(
                    std::find(b.ids.begin(), b.ids.end(), i) - b.ids.begin());
                const Q o{b.q[0], b.q[1], b.q[2], b.q[3]};
                const V3 p0 = b.p0[local];
                const Q r = qmul(qmul(o, Q{p0.x, p0.y, p0.z, 0.0f}), qinverse(o));
                const V3 np = add(b.pos, V3{r.x, r.y, r.z});
                x[i] = np.x;
                y[i] = np.y;
                z[i] = np.z;
                const V3 v = divs(sub(np, prev), static_cast<float>(static_cast<double>(dt)));
                vx[i] = v.x;
                vy[i] = v.y;
                vz[i] = v.z;
                reset_force(i);
            }
            else
            {
                if (mass[i] > 0.0f)
                {
                    const V3 a = mul(divs(V3{fx[i], fy[i], fz[i]}, mass[i]), dt);
                    vx[i] = vx[i] + a.x;
                    vy[i] = vy[i] + a.y;
                    vz[i] = vz[i] + a.z;
                }
                const float vit = norm3(vel(i));
                pe_kin[i] = static_cast<float>(0.5f * mass[i] * (vit * vit) * C_KINETIC);
                const V3 dx = mul(vel(i), dt);
                x[i] = x[i] + dx.x;
                y[i] = y[i] + dx.y;
                z[i] = z[i] + dx.z;
            }
            if (!std::isfinite(x[i]) || !std::isfinite(y[i]) || !std::isfinite(z[i]))
                finite = false;
            ke += pe_kin[i];
            reset_force(i);
        }
        energies[BS_ENERGY_KINETIC] += ke;
        update_grids();
        return finite;
    }

    bool step()
    {
        for (float & e : energies)
            e = 0.0f;
        if (cfg.spring_enable)
            compute_spring_forces();
        compute_particle_forces();
        if (rigid_on)
            solve_bodies();
        return update_positions();
    }

    // Rigid-body initialisation (RigidBody.cpp:57-123): total mass, mass-weighted
    // barycentre, local positions, spring states.
    void init_bodies(const std::vector<std::vector<int64_t>> & members)
    {
        bodies.clear();
        rigid.assign(n, 0);
        body_of.assign(n, 0);
        for (size_t b = 0; b < members.size(); ++b)
        {
            Body body;
            body.ids = members[b];
            double m = 0.;
            for (int64_t i : body.ids)
                m += mass[i];
            body.mass = m;
            V3 bary{0, 0, 0};
            double tm = 0.;
            for (int64_t i : body.ids)
            {
                bary = add(bary, mul(pos(i), mass[i]));
                tm = tm + mass[i];
            }
            if (!body.ids.empty())
                bary = mul(bary, static_cast<float>(1.0 / tm));
            body.pos = bary;
            for (int64_t i : body.ids)
                body.p0.push_back(sub(pos(i), body.pos));
            body.ibodyinv = 1.0 / ((2.0 / 5.0) * body.mass * 1.0 * 1.0);
            for (int64_t i : body.ids)
            {
                rigid[i] = 1;
                body_of[i] = static_cast<int32_t>(b);
            }
            bodies.push_back(body);
        }
        // Springs whose two ends are rigid become static (RigidBody.cpp:41-53).
        std::vector<int64_t> keep;
        for (int64_t s : dyn_springs)
            if (!(rigid[s_i[s]] && rigid[s_j[s]]))
                keep.push_back(s);
        dyn_springs = keep;
        rigid_on = true;
    }
};

} // namespace

extern "C" {

// The reference's default parameters (configuration::defaultConfiguration,
// src/configuration/Configuration.hpp:153-234) in the bs_config layout, restated here so that
// the oracle builds its configuration without the product library. Fields the reference does
// not have take the values that make the step the reference's: constant dielectric, the
// hard-coded membrane (src/forcefield/energy/imp.hpp:13-15), list rebuilt every 10 steps.
void bso_default_config(bs_config * c)
{
    std::memset(c, 0, sizeof(*c));
    c->nbsteps = -1;
    c->timestep = 0.01;
    c->neighborskin = 0.0;
    c->spring_enable = 0;
    c->spring_scale = 1.0;
    c->steric_enable = 0;
    c->steric_gridscale = 1.0;
    c->steric_cutoff = 1.0;
    c->steric_mode = BS_STERIC_LINEAR;
    c->coulomb_enable = 0;
    c->coulomb_scale = 1.0;
    c->coulomb_cutoff = 16.0;
    c->coulomb_dielectric = 1.0;
    c->hydrophobicity_enable = 0;
    c->hydrophobicity_scale = 1.0;
    c->hydrophobicity_cutoff = 15.0;
    c->impala_enable = 0;
    c->impala_scale = 1.0;
    c->viscosity_enable = 0;
    c->viscosity_value = 1.0;
    c->rigidbody_enable = 0;
    c->dielectric_mode = BS_DIELECTRIC_CONSTANT;
    c->impala_z0 = 15.75;
    c->impala_alpha = 1.99;
    c->rebuild_every = 10;
    c->list_skin = 1.0;
    c->probe_x = 1.0;
    c->probe_y = 1.0;
    c->probe_z = 1.0;
    c->probe_mass = 1.0;
    c->probe_epsilon = 1.0;
    c->probe_radius = 1.0;
    c->probe_charge = 0.0;
    c->potentialgrid_scale = 1.0;
    c->densitygrid_scale = 1.0;
}

void * bso_create(const bs_config * cfg, int64_t n, const float * xyz, const float * vel, const float * mass,
                  const float * charge, const float * radius, const float * eps, const float * hydro,
                  const float * sasa, const float * transfer, const uint8_t * is_static, int64_t ns,
                  const int32_t * ij, const float * r0, const float * k)
{
    auto * s = new Sim();
    s->cfg = *cfg;
    s->n = n;
    auto fill = [&](std::vector<float> & v, const float * src, float def) {
        v.assign(n, def);
        if (src)
            for (int64_t i = 0; i < n; ++i)
                v[i] = src[i];
    };
    s->x.resize(n);
    s->y.resize(n);
    s->z.resize(n);
    for (int64_t i = 0; i < n; ++i)
    {
        s->x[i] = xyz[3 * i];
        s->y[i] = xyz[3 * i + 1];
        s->z[i] = xyz[3 * i + 2];
    }
    s->vx.assign(n, 0);
    s->vy.assign(n, 0);
    s->vz.assign(n, 0);
    if (vel)
        for (int64_t i = 0; i < n; ++i)
        {
            s->vx[i] = vel[3 * i];
            s->vy[i] = vel[3 * i + 1];
            s->vz[i] = vel[3 * i + 2];
        }
    s->fx.assign(n, 0);
    s->fy.assign(n, 0);
    s->fz.assign(n, 0);
    fill(s->mass, mass, 1.0f);
    fill(s->charge, charge, 0.0f);
    fill(s->radius, radius, 1.0f);
    fill(s->eps, eps, 0.0f);
    fill(s->hydro, hydro, 0.0f);
    fill(s->sasa, sasa, 0.0f);
    fill(s->transfer, transfer, 0.0f);
    for (auto * v : {&s->pe_elec, &s->pe_steric, &s->pe_imp, &s->pe_hydro, &s->pe_kin})
        v->assign(n, 0.0f);
    s->is_static.assign(n, 0);
    if (is_static)
        for (int64_t i = 0; i < n; ++i)
            s->is_static[i] = is_static[i] ? 1 : 0;
    s->charged.assign(n, 0);
    s->hydrophobic.assign(n, 0);
    for (int64_t i = 0; i < n; ++i)
    {
        s->charged[i] = s->charge[i] != 0.0f;
        s->hydrophobic[i] = s->hydro[i] != 0.0f;
        if (!s->is_static[i])
            s->dynamic.push_back(i);
    }
    s->rigid.assign(n, 0);
    s->body_of.assign(n, 0);
    s->bonded.assign(n, {});
    for (int64_t t = 0; t < ns; ++t)
    {
        const int64_t a = ij[2 * t], b = ij[2 * t + 1];
        if (s->bonded[a].count(b))
            continue;
        const int64_t id = static_cast<int64_t>(s->s_i.size());
        s->s_i.push_back(a);
        s->s_j.push_back(b);
        s->s_r0.push_back(r0[t]);
        s->s_k.push_back(k[t]);
        s->s_energy.push_back(0.0f);
        s->bonded[a].insert(b);
        s->bonded[b].insert(a);
        if (!(s->is_static[a] && s->is_static[b]))
            s->dyn_springs.push_back(id);
    }
    FF & ff = s->ff;
    ff.mode = cfg->steric_mode;
    ff.stericscale = static_cast<float>(cfg->steric_gridscale);
    ff.coulombscale = static_cast<float>(cfg->coulomb_scale);
    ff.dielectric = static_cast<float>(cfg->coulomb_dielectric);
    ff.dielectric_mode = cfg->dielectric_mode;
    ff.springscale = static_cast<float>(cfg->spring_scale);
    ff.impscale = static_cast<float>(cfg->impala_scale);
    ff.hydroscale = static_cast<float>(cfg->hydrophobicity_scale);
    ff.imp_z0 = static_cast<float>(cfg->impala_z0);
    ff.imp_alpha = static_cast<float>(cfg->impala_alpha);
    // SpringNetwork::_setupProbe (SpringNetwork.cpp:749-766)
    s->probe_on = cfg->probe_enable != 0;
    s->probe.pos = {static_cast<float>(cfg->probe_x), static_cast<float>(cfg->probe_y), static_cast<float>(cfg->probe_z)};
    s->probe.vel = {0, 0, 0};
    s->probe.mass = static_cast<float>(cfg->probe_mass);
    s->probe.radius = static_cast<float>(cfg->probe_radius);
    s->probe.eps = static_cast<float>(cfg->probe_epsilon);
    s->probe.charge = static_cast<float>(cfg->probe_charge);
    s->setup_grids();
    return s;
}

// Field grid `which` (0 potential, 1 density) from its scalar values; used when the
// configuration enables it (potentialgrid.enable with coulomb.enable, densitygrid.enable).
void bso_set_field_grid(void * h, int32_t which, const int32_t * shape, const double * origin, const double * spacing,
                        const float * scalar)
{
    auto * s = static_cast<Sim *>(h);
    s->field[which].set(shape, origin, spacing, scalar);
    s->field[which].on = which == 0 ? s->cfg.potentialgrid_enable != 0 : s->cfg.densitygrid_enable != 0;
}

// The grid's cells, 4 floats each (scalar, force vector).
void bso_get_field_grid(void * h, int32_t which, float * out)
{
    const Field & f = static_cast<Sim *>(h)->field[which];
    for (size_t c = 0; c < f.sc.size(); ++c)
    {
        out[4 * c] = f.sc[c];
        out[4 * c + 1] = f.gx[c];
        out[4 * c + 2] = f.gy[c];
        out[4 * c + 3] = f.gz[c];
    }
}

// Per-particle burying (ParticleProperty::setBurying), caller order.
void bso_set_burying(void * h, const float * b)
{
    auto * s = static_cast<Sim *>(h);
    s->burying.assign(b, b + s->n);
}

// Probe position and velocity (float[6]); zeros when the probe is off.
void bso_get_probe(void * h, float * out)
{
    const auto * s = static_cast<const Sim *>(h);
    const float v[6] = {s->probe.pos.x, s->probe.pos.y, s->probe.pos.z, s->probe.vel.x, s->probe.vel.y, s->probe.vel.z};
    for (int k = 0; k < 6; ++k)
        out[k] = s->probe_on ? v[k] : 0.0f;
}

void bso_destroy(void * h) { delete static_cast<Sim *>(h); }

// The double membrane's offsets and tube curvatures (ForceField::setImpDoubleMembrane*).
void bso_set_membrane(void * h, float upper_offset, float lower_offset, float upper_curv, float lower_curv)
{
    auto * s = static_cast<Sim *>(h);
    s->ff.memb_uo = upper_offset;
    s->ff.memb_lo = lower_offset;
    s->ff.memb_uc = upper_curv;
    s->ff.memb_lc = lower_curv;
}

// Body b owns ids[offsets[b] .. offsets[b+1]).
int bso_set_rigid_bodies(void * h, int32_t nb, const int32_t * offsets, const int32_t * ids)
{
    auto * s = static_cast<Sim *>(h);
    std::vector<std::vector<int64_t>> members(nb);
    for (int32_t b = 0; b < nb; ++b)
        for (int32_t t = offsets[b]; t < offsets[b + 1]; ++t)
            members[b].push_back(ids[t]);
    s->init_bodies(members);
    return 0;
}

int bso_step(void * h, int32_t nsteps)
{
    auto * s = static_cast<Sim *>(h);
    for (int32_t t = 0; t < nsteps; ++t)
        if (!s->step())
            return BS_E_NONFINITE;
    return 0;
}

double bso_time_steps(void * h, int32_t nsteps)
{
    auto * s = static_cast<Sim *>(h);
    const auto t0 = std::chrono::steady_clock::now();
    for (int32_t t = 0; t < nsteps; ++t)
        s->step();
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

int bso_compute_forces(void * h)
{
    auto * s = static_cast<Sim *>(h);
    for (int64_t i = 0; i < s->n; ++i)
        s->reset_force(i);
    for (float & e : s->energies)
        e = 0.0f;
    if (s->cfg.spring_enable)
        s->compute_spring_forces();
    s->compute_particle_forces();
    return 0;
}

void bso_get_positions(void * h, float * out)
{
    auto * s = static_cast<Sim *>(h);
    for (int64_t i = 0; i < s->n; ++i)
    {
        out[3 * i] = s->x[i];
        out[3 * i + 1] = s->y[i];
        out[3 * i + 2] = s->z[i];
    }
}
void bso_get_velocities(void * h, float * out)
{
    auto * s = static_cast<Sim *>(h);
    for (int64_t i = 0; i < s->n; ++i)
    {
        out[3 * i] = s->vx[i];
        out[3 * i + 1] = s->vy[i];
        out[3 * i + 2] = s->vz[i];
    }
}
void bso_get_forces(void * h, float * out)
{
    auto * s = static_cast<Sim *>(h);
    for (int64_t i = 0; i < s->n; ++i)
    {
        out[3 * i] = s->fx[i];
        out[3 * i + 1] = s->fy[i];
        out[3 * i + 2] = s->fz[i];
    }
}
void bso_set_positions(void * h, const float * xyz)
{
    auto * s = static_cast<Sim *>(h);
    for (int64_t i = 0; i < s->n; ++i)
    {
        s->x[i] = xyz[3 * i];
        s->y[i] = xyz[3 * i + 1];
        s->z[i] = xyz[3 * i + 2];
    }
    s->setup_grids();
}
void bso_set_velocities(void * h, const float * v)
{
    auto * s = static_cast<Sim *>(h);
    for (int64_t i = 0; i < s->n; ++i)
    {
        s->vx[i] = v[3 * i];
        s->vy[i] = v[3 * i + 1];
        s->vz[i] = v[3 * i + 2];
    }
}
void bso_get_energies(void * h, double * out)
{
    auto * s = static_cast<Sim *>(h);
    for (int e = 0; e < BS_NUM_ENERGIES; ++e)
        out[e] = s->energies[e];
}

int64_t bso_get_pairs(void * h, int32_t term, int64_t * out, int64_t cap)
{
    auto * s = static_cast<Sim *>(h);
    const Grid & g = s->grid[term];
    if (!g.active)
        return 0;
    int64_t count = 0;
    for (int64_t i : s->dynamic)
    {
        if (term == BS_TERM_COULOMB && !s->charged[i])
            continue;
        if (term == BS_TERM_HYDROPHOBIC && !s->hydrophobic[i])
            continue;
        g.for_each_neighbor(i, s->x, s->y, s->z, [&](int64_t j) {
            if (!s->is_static[j] && j < i)
                return;
            if (s->cfg.spring_enable && s->bonded[i].count(j))
                return;
            const float d = norm3(sub(s->pos(j), s->pos(i)));
            if (!(d < g.cutoff))
                return;
            if (term != BS_TERM_STERIC && !(d != 0.0))
                return;
            if (count < cap)
            {
                out[2 * count] = std::min(i, j);
                out[2 * count + 1] = std::max(i, j);
            }
            ++count;
        });
    }
    return count;
}

int bso_get_cells(void * h, int32_t term, int64_t * out)
{
    auto * s = static_cast<Sim *>(h);
    Grid g = s->grid[term];
    for (int64_t i = 0; i < s->n; ++i)
        out[i] = -1;
    if (!g.active)
        return 0;
    g.build(s->x, s->y, s->z);
    if (g.included.empty())
        for (int64_t i = 0; i < s->n; ++i)
            out[i] = static_cast<int64_t>(g.cell_of(s->x[i], s->y[i], s->z[i]));
    else
        for (int64_t i : g.included)
            out[i] = static_cast<int64_t>(g.cell_of(s->x[i], s->y[i], s->z[i]));
    return 0;
}

// FP64 evaluation of the forces on dynamic particles and of the energies at the
// current positions, over the same pair set (exact double distances, no
// intermediate float rounding). Used to state the error of both the reference
// arithmetic and the device arithmetic against FP64.
int bso_eval_fp64(void * h, double * f_out, double * e_out)
{
    auto * s = static_cast<Sim *>(h);
    const int64_t n = s->n;
    const bs_config & c = s->cfg;
    std::vector<double> F(3 * n, 0.0);
    double E[BS_NUM_ENERGIES] = {0, 0, 0, 0, 0, 0};
    auto dvec = [&](int64_t i, int64_t j, double & dx, double & dy, double & dz) {
        dx = static_cast<double>(s->x[j]) - s->x[i];
        dy = static_cast<double>(s->y[j]) - s->y[i];
        dz = static_cast<double>(s->z[j]) - s->z[i];
    };
    if (c.spring_enable)
        for (int64_t sp : s->dyn_springs)
        {
            const int64_t a = s->s_i[sp], b = s->s_j[sp];
            if ((s->rigid[a] && s->rigid[b]) || (s->is_static[a] && s->is_static[b]))
                continue;
            double dx, dy, dz;
            dvec(a, b, dx, dy, dz);
            const double d = std::sqrt(dx * dx + dy * dy + dz * dz);
            const double k = s->s_k[sp], r0 = s->s_r0[sp], sc = s->ff.springscale;
            E[BS_ENERGY_SPRING] += sc * 0.5 * k * (d - r0) * (d - r0);
            const double m = sc * k * (d - r0) * C_SPRING_F;
            if (d > 0)
            {
                F[3 * a] += dx / d * m;
                F[3 * a + 1] += dy / d * m;
                F[3 * a + 2] += dz / d * m;
                F[3 * b] -= dx / d * m;
                F[3 * b + 1] -= dy / d * m;
                F[3 * b + 2] -= dz / d * m;
            }
        }
    auto term_pairs = [&](int term) {
        const Grid & g = s->grid[term];
        if (!g.active)
            return;
        for (int64_t i : s->dynamic)
        {
            if (term == BS_TERM_COULOMB && !s->charged[i])
                continue;
            if (term == BS_TERM_HYDROPHOBIC && !s->hydrophobic[i])
                continue;
            g.for_each_neighbor(i, s->x, s->y, s->z, [&](int64_t j) {
                if (!s->is_static[j] && j < i)
                    return;
                if (c.spring_enable && s->bonded[i].count(j))
                    return;
                const float df = norm3(sub(s->pos(j), s->pos(i)));
                if (!(df < g.cutoff))
                    return;
                if (term != BS_TERM_STERIC && !(df != 0.0))
                    return;
                double dx, dy, dz;
                dvec(i, j, dx, dy, dz);
                const double d = std::sqrt(dx * dx + dy * dy + dz * dz);
                double e = 0, m = 0;
                if (term == BS_TERM_STERIC)
                {
                    const double sc = s->ff.stericscale;
                    const double ri = s->radius[i], rj = s->radius[j], ei = s->eps[i], ej = s->eps[j];
                    if (c.steric_mode == BS_STERIC_LINEAR)
                    {
                        const double dv = d - (ri + rj);
                        if (dv <= 0)
                        {
                            e = 0.5 * dv * dv;
                            m = -std::fabs(dv) * C_SPRING_F;
                        }
                    }
                    else if (d >= C_MIN_DIST_VDW)
                    {
                        if (c.steric_mode == BS_STERIC_LJ_12_6_AMBER)
                        {
                            const double eij = std::sqrt(ei * ej), rij = std::sqrt(ri * rj), q = rij / d;
                            e = eij * (std::pow(q, 12) - 2.0 * std::pow(q, 6));
                            m = 12.0 * eij * (std::pow(q, 6) - std::pow(q, 12)) / d * C_SPRING_F;
                        }
                        else if (c.steric_mode == BS_STERIC_LJ_8_6_LEWITT)
                        {
                            const double eij = std::sqrt(ei * ej), rij = std::sqrt(ri * rj), q = rij / d;
                            e = eij * (3.0 * std::pow(q, 8) - 4.0 * std::pow(q, 6));
                            m = 24.0 * eij * (std::pow(q, 6) - std::pow(q, 8)) / d * C_SPRING_F;
                        }
                        else
                        {
                            const double eij = ei * ej, rij = ri * rj, q = rij / d;
                            e = eij * (std::pow(q, 8) - std::pow(q, 6));
                            m = eij * (6.0 * std::pow(q, 6) - 8.0 * std::pow(q, 8)) / d * C_SPRING_F;
                        }
                    }
                    e *= sc;
                    m *= sc;
                }
                else if (term == BS_TERM_COULOMB)
                {
                    const double sc = s->ff.coulombscale, D = s->ff.dielectric;
                    const double qq = static_cast<double>(s->charge[i]) * s->charge[j];
                    if (d >= C_MIN_DIST_ELEC)
                    {
                        const double epsr = c.dielectric_mode == BS_DIELECTRIC_DISTANCE ? D * d : D;
                        e = C_COULOMB_K * qq * C_ELECTRONCHARGE_TO_COULOMB * C_ELECTRONCHARGE_TO_COULOMB /
                            (epsr * d * C_ANGSTROM_TO_METER) * C_AVOGADRO * 1e-3;
                        const double mult = c.dielectric_mode == BS_DIELECTRIC_DISTANCE ? 2.0 : 1.0;
                        m = -mult * qq / (4.0 * C_PI * epsr * d * d) * C_ELEC_F;
                    }
                    e *= sc;
                    m *= sc;
                }
                else
                {
                    const double sc = s->ff.hydroscale;
                    const double hh = static_cast<double>(s->hydro[i]) * s->hydro[j];
                    e = -hh * std::exp(-d) * C_AVOGADRO * 1e-3 * sc;
                    m = hh * std::exp(-d) * C_SPRING_F * sc;
                }
                const int slot = term == BS_TERM_STERIC ? BS_ENERGY_STERIC
                                 : term == BS_TERM_COULOMB ? BS_ENERGY_ELECTROSTATIC
                                                           : BS_ENERGY_HYDROPHOBIC;
                E[slot] += e;
                if (d > 0)
                {
                    F[3 * i] += dx / d * m;
                    F[3 * i + 1] += dy / d * m;
                    F[3 * i + 2] += dz / d * m;
                    if (!s->is_static[j])
                    {
                        F[3 * j] -= dx / d * m;
                        F[3 * j + 1] -= dy / d * m;
                        F[3 * j + 2] -= dz / d * m;
                    }
                }
            });
        }
    };
    if (c.coulomb_enable)
        term_pairs(BS_TERM_COULOMB);
    if (c.steric_enable)
        term_pairs(BS_TERM_STERIC);
    if (c.hydrophobicity_enable)
        term_pairs(BS_TERM_HYDROPHOBIC);
    for (int64_t i : s->dynamic)
    {
        if (c.viscosity_enable)
        {
            F[3 * i] -= static_cast<double>(s->vx[i]) * c.viscosity_value;
            F[3 * i + 1] -= static_cast<double>(s->vy[i]) * c.viscosity_value;
            F[3 * i + 2] -= static_cast<double>(s->vz[i]) * c.viscosity_value;
        }
        if (c.impala_enable && !s->ff.flat())
        {
            // double membrane in FP64: each membrane's depth and direction from its tube axis
            const double S = s->sasa[i], T = s->transfer[i];
            const double a = static_cast<float>(c.impala_alpha), z0 = static_cast<float>(c.impala_z0);
            const double offs[2] = {s->ff.memb_uo, -static_cast<double>(s->ff.memb_lo)};
            const double curv[2] = {s->ff.memb_uc, s->ff.memb_lc};
            for (int m = 0; m < 2; ++m)
            {
                const double R = curv[m] == 0.0 ? 1.0e6 : std::fabs(1.0 / curv[m]);
                const int sg = (curv[m] > 0.0) - (curv[m] < 0.0);
                const double cz_axis = offs[m] - sg * R;
                const double rx = s->x[i], rz = s->z[i] - cz_axis, rn = std::sqrt(rx * rx + rz * rz);
                const double depth = sg == 0 ? static_cast<double>(s->z[i])
                                             : (s->z[i] > cz_axis ? sg * rn : -sg * rn) + offs[m] - R;
                const double u = depth - offs[m];
                const double ex = std::exp(a * (std::fabs(u) - z0));
                E[BS_ENERGY_IMP] += s->ff.impscale * (-S * T + C_ALIP * S) * (0.5 - 1.0 / (1.0 + ex));
                double dcz = a * u * ex / ((ex + 1) * (ex + 1) * std::fabs(u));
                if (!std::isfinite(dcz))
                    dcz = 0.0;
                double dx = 0.0, dz = 1.0;
                if (sg != 0)
                {
                    dx = rn > 0.0 ? rx / rn : 0.0;
                    dz = rn > 0.0 ? rz / rn : 0.0;
                }
                const double f = s->ff.impscale * (-S * T + C_ALIP * S) * dcz * C_IMP_F;
                F[3 * i] -= f * dx;
                F[3 * i + 2] -= f * dz;
            }
        }
        else if (c.impala_enable)
        {
            const double zz = s->z[i], S = s->sasa[i], T = s->transfer[i];
            const double a = static_cast<float>(c.impala_alpha), z0 = static_cast<float>(c.impala_z0);
            const double ex = std::exp(a * (std::fabs(zz) - z0));
            const double cz = 0.5 - 1.0 / (1.0 + ex);
            E[BS_ENERGY_IMP] += s->ff.impscale * (-S * T + C_ALIP * S) * cz;
            double dcz = a * zz * ex / ((ex + 1) * (ex + 1) * std::fabs(zz));
            if (!std::isfinite(dcz))
                dcz = 0.0;
            F[3 * i + 2] -= s->ff.impscale * (-S * T + C_ALIP * S) * dcz * C_IMP_F;
        }
    }
    for (int64_t i = 0; i < n; ++i)
    {
        if (s->is_static[i])
            continue;
        f_out[3 * i] = F[3 * i];
        f_out[3 * i + 1] = F[3 * i + 1];
        f_out[3 * i + 2] = F[3 * i + 2];
    }
    for (int e = 0; e < BS_NUM_ENERGIES; ++e)
        e_out[e] = E[e];
    return 0;
}

} // extern "C"
