// adjoint_fp64.cpp -- TEST INFRASTRUCTURE ONLY: FP64 reference for the gradient path.
// Only tests/ and bench.py's checks load it (through libbs_oracle.so); the product never does.
//
// It restates, in double precision, the damped dynamics the CUDA step integrates
// (src/spn/SpringNetwork.cpp:63-241, src/spn/Particle.cpp:80-128, 368-429,
// src/forcefield/energy/spring.hpp:17-29, steric.hpp:37-59): spring forces, linear steric
// overlap forces between pairs that are not spring-bonded, viscosity from the pre-step velocity,
// then v += F/m dt (when m > 0) and x += v dt; static particles never move. On top of it:
//   bso_loss_fp64      L = (1/n) sum_i |x_i(N) - target_i|^2
//   bso_adjoint_fp64   L and dL/dk, dL/dr0 of every spring by the discrete adjoint (all states
//                      kept, no checkpoints), the FP64 reference gradient
//   bso_fd_fp64        central finite differences of L for selected springs (OpenMP over the
//                      selected springs), the check of bso_adjoint_fp64 itself; the difference
//                      of the two losses is formed from the two final states, not by subtracting
//                      two nearly equal losses
// Coulomb pairs (Particle.cpp:191-253, electrostatic.hpp:16-49) join the forces when enabled:
// F_i = phi(d) u with phi = -C q_i q_j / d^2 (constant dielectric) or -2 C q_i q_j / d^3 (eps = D r),
// for pairs of charged particles closer than the cutoff and at least 0.001 A apart; the adjoint
// also returns dL/dq of every particle (a pair with one charge zero still has a charge gradient).
// This gradient path has no counterpart in the reference; the forward dynamics it
// differentiates is the restated reference step, so parity of the forward is pinned through the
// step oracle and the gradient is pinned by finite differences.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <unordered_map>
#include <unordered_set>
#include <vector>

namespace
{

// unit conversion of spring-like forces, kJ/mol/A -> Da.A.fs^-2 (constants.hpp:88-105)
const double kNewtonToDaAFs2 = 1.0E10 * (1.0 / 1.66054E-27) * 1.0E-15 * 1.0E-15;
const double kSpringF = 1.0E3 / 6.02214169E23 * 1.0E10 * kNewtonToDaAFs2;
// Coulomb force of two unit charges at 1 A with dielectric 1, Da.A.fs^-2 (constants.hpp:110-118)
const double kElecF = kNewtonToDaAFs2 * (1.60217653E-19 * 1.60217653E-19) / (8.854187817E-12 * 1.0E-10 * 1.0E-10) /
                      (4.0 * 3.1415927);

struct Model
{
    int64_t n = 0;
    // Positions are carried as x0 + delta: x0 (the start, exact floats) never changes and delta
    // is the displacement, so separations and the loss keep the precision of the displacement
    // (1e-16 of a few A) instead of that of a coordinate (1e-16 of ~50 A).
    std::vector<double> x0;
    std::vector<double> mass, radius;
    std::vector<uint8_t> fixed;
    std::vector<int32_t> si, sj;
    std::vector<double> k, r0;
    double dt = 0.01, spring_scale = 1.0, steric_cutoff = 8.0, steric_scale = 1.0, visc = 0.0;
    bool spring_on = true, steric_on = false, visc_on = false;
    // Coulomb: charges, cutoff, C = conversion * scale / D, distance-dependent dielectric
    std::vector<double> q;
    bool coul_on = false, coul_dist = false;
    double coul_cutoff = 12.0, coul_c = 0.0;
    std::unordered_set<uint64_t> bonded;
    double max_radius = 0.0;

    static uint64_t key(int64_t a, int64_t b)
    {
        return (static_cast<uint64_t>(std::min(a, b)) << 32) | static_cast<uint64_t>(std::max(a, b));
    }

    // separation x_j - x_i for displacements `dl`
    void sep(const std::vector<double> & dl, int64_t i, int64_t j, double u[3]) const
    {
        for (int c = 0; c < 3; ++c)
            u[c] = (x0[3 * j + c] - x0[3 * i + c]) + (dl[3 * j + c] - dl[3 * i + c]);
    }

    // Linear steric pairs (i < j, not bonded when springs are on) with d < cutoff and
    // d < r_i + r_j: only overlapping pairs carry a force, so the search radius is the smaller
    // of the cutoff and the largest contact distance.
    void steric_pairs(const std::vector<double> & dl, std::vector<std::pair<int64_t, int64_t>> & out) const
    {
        std::vector<double> x(3 * n);
        for (int64_t i = 0; i < 3 * n; ++i)
            x[i] = x0[i] + dl[i];
        out.clear();
        const double reach = std::min(steric_cutoff, 2.0 * max_radius);
        if (!(reach > 0.0) || n < 2)
            return;
        double lo[3] = {1e300, 1e300, 1e300};
        for (int64_t i = 0; i < n; ++i)
            for (int c = 0; c < 3; ++c)
                lo[c] = std::min(lo[c], x[3 * i + c]);
        std::unordered_map<int64_t, std::vector<int64_t>> cells;
        auto cid = [&](int64_t a, int64_t b, int64_t c) { return (a * 2000003LL + b) * 2000003LL + c; };
        std::vector<int64_t> cc(3 * n);
        for (int64_t i = 0; i < n; ++i)
        {
            for (int c = 0; c < 3; ++c)
                cc[3 * i + c] = static_cast<int64_t>(std::floor((x[3 * i + c] - lo[c]) / reach));
            cells[cid(cc[3 * i], cc[3 * i + 1], cc[3 * i + 2])].push_back(i);
        }
        for (int64_t i = 0; i < n; ++i)
            for (int64_t dz = -1; dz <= 1; ++dz)
                for (int64_t dy = -1; dy <= 1; ++dy)
                    for (int64_t dx = -1; dx <= 1; ++dx)
                    {
                        auto it = cells.find(cid(cc[3 * i] + dx, cc[3 * i + 1] + dy, cc[3 * i + 2] + dz));
                        if (it == cells.end())
                            continue;
                        for (int64_t j : it->second)
                        {
                            if (j <= i || (fixed[i] && fixed[j]))
                                continue;
                            if (spring_on && bonded.count(key(i, j)))
                                continue;
                            double a3[3];
                            sep(dl, i, j, a3);
                            const double d = std::sqrt(a3[0] * a3[0] + a3[1] * a3[1] + a3[2] * a3[2]);
                            if (d < steric_cutoff && d < radius[i] + radius[j] && d > 0.0)
                                out.emplace_back(i, j);
                        }
                    }
    }

    // Pairs (i < j, not both static, not bonded when springs are on) closer than the Coulomb cutoff
    // and at least 0.001 A apart, with at least one charge (all = true) or both charges (all =
    // false) non-zero.
    void coulomb_pairs(const std::vector<double> & dl, const std::vector<double> & qq, bool all,
                       std::vector<std::pair<int64_t, int64_t>> & out) const
    {
        out.clear();
        if (!coul_on || n < 2)
            return;
        std::vector<double> x(3 * n);
        for (int64_t i = 0; i < 3 * n; ++i)
            x[i] = x0[i] + dl[i];
        double lo[3] = {1e300, 1e300, 1e300};
        for (int64_t i = 0; i < n; ++i)
            for (int c = 0; c < 3; ++c)
                lo[c] = std::min(lo[c], x[3 * i + c]);
        std::unordered_map<int64_t, std::vector<int64_t>> cells;
        auto cid = [&](int64_t a, int64_t b, int64_t c) { return (a * 2000003LL + b) * 2000003LL + c; };
        std::vector<int64_t> cc(3 * n);
        for (int64_t i = 0; i < n; ++i)
        {
            for (int c = 0; c < 3; ++c)
                cc[3 * i + c] = static_cast<int64_t>(std::floor((x[3 * i + c] - lo[c]) / coul_cutoff));
            cells[cid(cc[3 * i], cc[3 * i + 1], cc[3 * i + 2])].push_back(i);
        }
        for (int64_t i = 0; i < n; ++i)
            for (int64_t dz = -1; dz <= 1; ++dz)
                for (int64_t dy = -1; dy <= 1; ++dy)
                    for (int64_t dx = -1; dx <= 1; ++dx)
                    {
                        auto it = cells.find(cid(cc[3 * i] + dx, cc[3 * i + 1] + dy, cc[3 * i + 2] + dz));
                        if (it == cells.end())
                            continue;
                        for (int64_t j : it->second)
                        {
                            if (j <= i || (fixed[i] && fixed[j]))
                                continue;
                            const bool qi = qq[i] != 0.0, qj = qq[j] != 0.0;
                            if (all ? !(qi || qj) : !(qi && qj))
                                continue;
                            if (spring_on && bonded.count(key(i, j)))
                                continue;
                            double a3[3];
                            sep(dl, i, j, a3);
                            const double d = std::sqrt(a3[0] * a3[0] + a3[1] * a3[1] + a3[2] * a3[2]);
                            if (d < coul_cutoff && d >= 0.001)
                                out.emplace_back(i, j);
                        }
                    }
    }

    // Coulomb force along u (on i, towards j) and its d-derivative, and the same per unit charge of
    // i (phi / q_i) and of j (phi / q_j), for charges qi, qj at distance d.
    void coulomb_phi(double qi, double qj, double d, double & phi, double & dphi, double & per_i, double & per_j) const
    {
        if (coul_dist)
        {
            const double d3 = d * d * d;
            per_i = -2.0 * coul_c * qj / d3;
            per_j = -2.0 * coul_c * qi / d3;
            phi = per_i * qi;
            dphi = -3.0 * phi / d;
        }
        else
        {
            const double d2 = d * d;
            per_i = -coul_c * qj / d2;
            per_j = -coul_c * qi / d2;
            phi = per_i * qi;
            dphi = -2.0 * phi / d;
        }
    }

    // Conservative forces at positions x (forces on static particles are computed but unused).
    void forces(const std::vector<double> & dl, const std::vector<double> & kk, const std::vector<double> & rr,
                const std::vector<double> & qq, std::vector<double> & f,
                std::vector<std::pair<int64_t, int64_t>> & pairs) const
    {
        std::fill(f.begin(), f.end(), 0.0);
        if (spring_on)
            for (size_t t = 0; t < si.size(); ++t)
            {
                const int64_t a = si[t], b = sj[t];
                double u3[3];
                sep(dl, a, b, u3);
                const double ux = u3[0], uy = u3[1], uz = u3[2];
                const double d = std::sqrt(ux * ux + uy * uy + uz * uz);
                if (!(d > 0.0))
                    continue;
                const double phi = kSpringF * spring_scale * kk[t] * (d - rr[t]) / d;
                f[3 * a] += phi * ux;
                f[3 * a + 1] += phi * uy;
                f[3 * a + 2] += phi * uz;
                f[3 * b] -= phi * ux;
                f[3 * b + 1] -= phi * uy;
                f[3 * b + 2] -= phi * uz;
            }
        pairs.clear();
        if (steric_on)
        {
            steric_pairs(dl, pairs);
            for (const auto & pr : pairs)
            {
                const int64_t a = pr.first, b = pr.second;
                double u3[3];
                sep(dl, a, b, u3);
                const double ux = u3[0], uy = u3[1], uz = u3[2];
                const double d = std::sqrt(ux * ux + uy * uy + uz * uz);
                const double phi = kSpringF * steric_scale * (d - (radius[a] + radius[b])) / d;
                f[3 * a] += phi * ux;
                f[3 * a + 1] += phi * uy;
                f[3 * a + 2] += phi * uz;
                f[3 * b] -= phi * ux;
                f[3 * b + 1] -= phi * uy;
                f[3 * b + 2] -= phi * uz;
            }
        }
        if (coul_on)
        {
            std::vector<std::pair<int64_t, int64_t>> cp;
            coulomb_pairs(dl, qq, false, cp);
            for (const auto & pr : cp)
            {
                const int64_t a = pr.first, b = pr.second;
                double u3[3];
                sep(dl, a, b, u3);
                const double d = std::sqrt(u3[0] * u3[0] + u3[1] * u3[1] + u3[2] * u3[2]);
                double phi, dphi, pa, pb;
                coulomb_phi(qq[a], qq[b], d, phi, dphi, pa, pb);
                for (int c = 0; c < 3; ++c)
                {
                    f[3 * a + c] += phi * u3[c] / d;
                    f[3 * b + c] -= phi * u3[c] / d;
                }
            }
        }
    }

    // N steps from (x0, v); returns the final displacements, keeping the start-of-step
    // displacements and steric pairs when `keep` is non-null.
    void run(std::vector<double> v, const std::vector<double> & kk, const std::vector<double> & rr,
             const std::vector<double> & qq, int nsteps, std::vector<double> & xf,
             std::vector<std::vector<double>> * keep,
             std::vector<std::vector<std::pair<int64_t, int64_t>>> * keep_pairs) const
    {
        std::vector<double> x(3 * n, 0.0);
        std::vector<double> f(3 * n);
        std::vector<std::pair<int64_t, int64_t>> pairs;
        for (int s = 0; s < nsteps; ++s)
        {
            if (keep)
                (*keep)[s] = x;
            forces(x, kk, rr, qq, f, pairs);
            if (keep_pairs)
                (*keep_pairs)[s] = pairs;
            for (int64_t i = 0; i < n; ++i)
            {
                if (fixed[i])
                    continue;
                for (int c = 0; c < 3; ++c)
                {
                    double fc = f[3 * i + c];
                    if (visc_on)
                        fc -= visc * v[3 * i + c];
                    if (mass[i] > 0.0)
                        v[3 * i + c] += fc / mass[i] * dt;
                    x[3 * i + c] += v[3 * i + c] * dt;
                }
            }
        }
        xf = x;
    }

    double loss(const std::vector<double> & dl, const std::vector<double> & target) const
    {
        double l = 0.0;
        for (int64_t i = 0; i < 3 * n; ++i)
        {
            const double e = (x0[i] - target[i]) + dl[i];
            l += e * e;
        }
        return l / static_cast<double>(n);
    }
};

Model make_model(int64_t n, const float * mass, const float * radius, const uint8_t * is_static, int64_t ns,
                 const int32_t * ij, const float * k, const float * r0, double dt, int spring_on, double spring_scale,
                 int steric_on, double steric_cutoff, double steric_scale, int visc_on, double visc,
                 const float * charge, int coul_on, double coul_cutoff, double coul_c, int coul_dist)
{
    Model m;
    m.n = n;
    m.mass.assign(n, 1.0);
    m.radius.assign(n, 1.0);
    m.fixed.assign(n, 0);
    for (int64_t i = 0; i < n; ++i)
    {
        if (mass)
            m.mass[i] = mass[i];
        if (radius)
            m.radius[i] = radius[i];
        if (is_static)
            m.fixed[i] = is_static[i] ? 1 : 0;
        m.max_radius = std::max(m.max_radius, m.radius[i]);
    }
    for (int64_t t = 0; t < ns; ++t)
    {
        const uint64_t key = Model::key(ij[2 * t], ij[2 * t + 1]);
        if (!m.bonded.insert(key).second)
            continue; // repeated pair: ignored, as when springs are added
        m.si.push_back(ij[2 * t]);
        m.sj.push_back(ij[2 * t + 1]);
        m.k.push_back(k[t]);
        m.r0.push_back(r0[t]);
    }
    m.dt = dt;
    m.spring_on = spring_on != 0;
    m.spring_scale = spring_scale;
    m.steric_on = steric_on != 0;
    m.steric_cutoff = steric_cutoff;
    m.steric_scale = steric_scale;
    m.visc_on = visc_on != 0;
    m.visc = visc;
    m.q.assign(n, 0.0);
    if (charge)
        for (int64_t i = 0; i < n; ++i)
            m.q[i] = charge[i];
    m.coul_on = coul_on != 0;
    m.coul_cutoff = coul_cutoff;
    m.coul_c = coul_c;
    m.coul_dist = coul_dist != 0;
    return m;
}

std::vector<double> to_d(const float * a, int64_t count, double def = 0.0)
{
    std::vector<double> out(count, def);
    if (a)
        for (int64_t i = 0; i < count; ++i)
            out[i] = a[i];
    return out;
}

} // namespace

extern "C" {

double bso_loss_fp64(int64_t n, const float * xyz, const float * vel, const float * mass, const float * radius,
                     const uint8_t * is_static, int64_t ns, const int32_t * ij, const float * k, const float * r0,
                     double dt, int spring_on, double spring_scale, int steric_on, double steric_cutoff,
                     double steric_scale, int visc_on, double visc, const float * charge, int coul_on,
                     double coul_cutoff, double coul_c, int coul_dist, int32_t nsteps, const float * target)
{
    Model m = make_model(n, mass, radius, is_static, ns, ij, k, r0, dt, spring_on, spring_scale, steric_on,
                         steric_cutoff, steric_scale, visc_on, visc, charge, coul_on, coul_cutoff, coul_c, coul_dist);
    m.x0 = to_d(xyz, 3 * n);
    std::vector<double> xf;
    m.run(to_d(vel, 3 * n), m.k, m.r0, m.q, nsteps, xf, nullptr, nullptr);
    return m.loss(xf, to_d(target, 3 * n));
}

// Discrete adjoint in FP64 (same equations as the device sweep, all states kept). dL_dk and
// dL_dr0 have one entry per distinct spring, in upload order.
int bso_adjoint_fp64(int64_t n, const float * xyz, const float * vel, const float * mass, const float * radius,
                     const uint8_t * is_static, int64_t ns, const int32_t * ij, const float * k, const float * r0,
                     double dt, int spring_on, double spring_scale, int steric_on, double steric_cutoff,
                     double steric_scale, int visc_on, double visc, const float * charge, int coul_on,
                     double coul_cutoff, double coul_c, int coul_dist, int32_t nsteps, const float * target,
                     double * loss, double * dL_dk, double * dL_dr0, double * dL_dq)
{
    Model m = make_model(n, mass, radius, is_static, ns, ij, k, r0, dt, spring_on, spring_scale, steric_on,
                         steric_cutoff, steric_scale, visc_on, visc, charge, coul_on, coul_cutoff, coul_c, coul_dist);
    m.x0 = to_d(xyz, 3 * n);
    std::vector<std::vector<double>> xs(nsteps);
    std::vector<std::vector<std::pair<int64_t, int64_t>>> ps(nsteps);
    std::vector<double> xf;
    m.run(to_d(vel, 3 * n), m.k, m.r0, m.q, nsteps, xf, &xs, &ps);
    std::vector<double> gq(n, 0.0);
    const std::vector<double> tg = to_d(target, 3 * n);
    *loss = m.loss(xf, tg);
    const size_t nsp = m.si.size();
    std::vector<double> gk(nsp, 0.0), gr(nsp, 0.0);
    std::vector<double> lx(3 * n, 0.0), lv(3 * n, 0.0), nu(3 * n, 0.0), h(3 * n, 0.0);
    std::vector<double> a(n, 1.0), b(n, 0.0);
    for (int64_t i = 0; i < n; ++i)
    {
        if (m.fixed[i])
            continue;
        if (m.mass[i] > 0.0)
        {
            b[i] = dt / m.mass[i];
            a[i] = m.visc_on ? 1.0 - m.visc * dt / m.mass[i] : 1.0;
        }
        for (int c = 0; c < 3; ++c)
            lx[3 * i + c] = 2.0 * ((m.x0[3 * i + c] - tg[3 * i + c]) + xf[3 * i + c]) / static_cast<double>(n);
    }
    for (int s = nsteps - 1; s >= 0; --s)
    {
        const std::vector<double> & x = xs[s];
        for (int64_t i = 0; i < n; ++i)
            for (int c = 0; c < 3; ++c)
                nu[3 * i + c] = b[i] * (lv[3 * i + c] + dt * lx[3 * i + c]);
        std::fill(h.begin(), h.end(), 0.0);
        // pair (i, j) with w = nu_j - nu_i: row i gets H w, row j gets H (nu_i - nu_j) = -H w
        auto add_pair = [&](int64_t i, int64_t j, double phi, double dphi) {
            double s3[3];
            m.sep(x, i, j, s3);
            const double ux0 = s3[0], uy0 = s3[1], uz0 = s3[2];
            const double d = std::sqrt(ux0 * ux0 + uy0 * uy0 + uz0 * uz0);
            if (!(d > 0.0))
                return;
            const double u[3] = {ux0 / d, uy0 / d, uz0 / d};
            const double w[3] = {nu[3 * j] - nu[3 * i], nu[3 * j + 1] - nu[3 * i + 1], nu[3 * j + 2] - nu[3 * i + 2]};
            const double uw = u[0] * w[0] + u[1] * w[1] + u[2] * w[2];
            for (int c = 0; c < 3; ++c)
            {
                const double hw = dphi * uw * u[c] + phi / d * (w[c] - uw * u[c]);
                h[3 * i + c] += hw;
                h[3 * j + c] -= hw;
            }
        };
        if (m.spring_on)
            for (size_t t = 0; t < nsp; ++t)
            {
                const int64_t i = m.si[t], j = m.sj[t];
                double s3[3];
                m.sep(x, i, j, s3);
                const double ux0 = s3[0], uy0 = s3[1], uz0 = s3[2];
                const double d = std::sqrt(ux0 * ux0 + uy0 * uy0 + uz0 * uz0);
                if (!(d > 0.0))
                    continue;
                const double cs = kSpringF * m.spring_scale;
                add_pair(i, j, cs * m.k[t] * (d - m.r0[t]), cs * m.k[t]);
                // dF_i/dk = cs (d - r0) u, dF_j/dk = -cs (d - r0) u; dF/dr0 = -cs k u (and +)
                double un = 0.0;
                for (int c = 0; c < 3; ++c)
                    un += s3[c] / d * (nu[3 * i + c] - nu[3 * j + c]);
                gk[t] += cs * (d - m.r0[t]) * un;
                gr[t] -= cs * m.k[t] * un;
            }
        if (m.steric_on)
            for (const auto & pr : ps[s])
            {
                const int64_t i = pr.first, j = pr.second;
                double s3[3];
                m.sep(x, i, j, s3);
                const double ux0 = s3[0], uy0 = s3[1], uz0 = s3[2];
                const double d = std::sqrt(ux0 * ux0 + uy0 * uy0 + uz0 * uz0);
                const double cs = kSpringF * m.steric_scale;
                add_pair(i, j, cs * (d - (m.radius[i] + m.radius[j])), cs);
            }
        if (m.coul_on)
        {
            // every pair with a charge: forces for both charged, charge gradients for either
            std::vector<std::pair<int64_t, int64_t>> cp;
            m.coulomb_pairs(x, m.q, true, cp);
            for (const auto & pr : cp)
            {
                const int64_t i = pr.first, j = pr.second;
                double s3[3];
                m.sep(x, i, j, s3);
                const double d = std::sqrt(s3[0] * s3[0] + s3[1] * s3[1] + s3[2] * s3[2]);
                double phi, dphi, per_i, per_j;
                m.coulomb_phi(m.q[i], m.q[j], d, phi, dphi, per_i, per_j);
                if (m.q[i] != 0.0 && m.q[j] != 0.0)
                    add_pair(i, j, phi, dphi);
                // dF_i/dq = (phi / q) u, dF_j/dq = -(phi / q) u
                double un = 0.0;
                for (int c = 0; c < 3; ++c)
                    un += s3[c] / d * (nu[3 * i + c] - nu[3 * j + c]);
                gq[i] += per_i * un;
                gq[j] += per_j * un;
            }
        }
        for (int64_t i = 0; i < n; ++i)
        {
            if (m.fixed[i])
            {
                for (int c = 0; c < 3; ++c)
                    lx[3 * i + c] = lv[3 * i + c] = 0.0;
                continue;
            }
            for (int c = 0; c < 3; ++c)
            {
                const double mu = lv[3 * i + c] + dt * lx[3 * i + c];
                lx[3 * i + c] += h[3 * i + c];
                lv[3 * i + c] = a[i] * mu;
            }
        }
    }
    for (size_t t = 0; t < nsp; ++t)
    {
        dL_dk[t] = gk[t];
        dL_dr0[t] = gr[t];
    }
    if (dL_dq)
        for (int64_t i = 0; i < n; ++i)
            dL_dq[i] = gq[i];
    return 0;
}

// Central differences (h relative to each parameter's magnitude, at least h absolute) of L with
// respect to the stiffness and rest length of the selected springs.
int bso_fd_fp64(int64_t n, const float * xyz, const float * vel, const float * mass, const float * radius,
                const uint8_t * is_static, int64_t ns, const int32_t * ij, const float * k, const float * r0, double dt,
                int spring_on, double spring_scale, int steric_on, double steric_cutoff, double steric_scale,
                int visc_on, double visc, const float * charge, int coul_on, double coul_cutoff, double coul_c,
                int coul_dist, int32_t nsteps, const float * target, int64_t nsel, const int64_t * sel, double h,
                double * fd_k, double * fd_r0)
{
    Model m = make_model(n, mass, radius, is_static, ns, ij, k, r0, dt, spring_on, spring_scale, steric_on,
                         steric_cutoff, steric_scale, visc_on, visc, charge, coul_on, coul_cutoff, coul_c, coul_dist);
    m.x0 = to_d(xyz, 3 * n);
    const std::vector<double> v0 = to_d(vel, 3 * n), tg = to_d(target, 3 * n);
#pragma omp parallel for schedule(dynamic)
    for (int64_t q = 0; q < 2 * nsel; ++q)
    {
        const int64_t t = sel[q / 2];
        const bool is_k = (q % 2) == 0;
        std::vector<double> kk = m.k, rr = m.r0;
        std::vector<double> & p = is_k ? kk : rr;
        const double step = h * std::max(1.0, std::fabs(p[t]));
        const double p0 = p[t];
        std::vector<double> xp, xm;
        p[t] = p0 + step;
        m.run(v0, kk, rr, m.q, nsteps, xp, nullptr, nullptr);
        p[t] = p0 - step;
        m.run(v0, kk, rr, m.q, nsteps, xm, nullptr, nullptr);
        // L+ - L- as sum (x+ - x-) . (x+ + x- - 2 target) / n: the two losses agree to ~1e-12
        // relative, so subtracting them would leave mostly their rounding
        double dl = 0.0;
        for (int64_t i = 0; i < 3 * n; ++i)
            dl += (xp[i] - xm[i]) * (2.0 * (m.x0[i] - tg[i]) + xp[i] + xm[i]);
        (is_k ? fd_k : fd_r0)[q / 2] = dl / static_cast<double>(n) / (2.0 * step);
    }
    return 0;
}

// Central differences of L with respect to the charges of the selected particles (step h absolute;
// a zero charge becomes +-h, which adds its pairs with the O(h) forces they then carry).
int bso_fd_q_fp64(int64_t n, const float * xyz, const float * vel, const float * mass, const float * radius,
                  const uint8_t * is_static, int64_t ns, const int32_t * ij, const float * k, const float * r0,
                  double dt, int spring_on, double spring_scale, int steric_on, double steric_cutoff,
                  double steric_scale, int visc_on, double visc, const float * charge, int coul_on,
                  double coul_cutoff, double coul_c, int coul_dist, int32_t nsteps, const float * target, int64_t nsel,
                  const int64_t * sel, double h, double * fd_q)
{
    Model m = make_model(n, mass, radius, is_static, ns, ij, k, r0, dt, spring_on, spring_scale, steric_on,
                         steric_cutoff, steric_scale, visc_on, visc, charge, coul_on, coul_cutoff, coul_c, coul_dist);
    m.x0 = to_d(xyz, 3 * n);
    const std::vector<double> v0 = to_d(vel, 3 * n), tg = to_d(target, 3 * n);
#pragma omp parallel for schedule(dynamic)
    for (int64_t t = 0; t < nsel; ++t)
    {
        const int64_t i = sel[t];
        std::vector<double> qq = m.q;
        std::vector<double> xp, xm;
        qq[i] = m.q[i] + h;
        m.run(v0, m.k, m.r0, qq, nsteps, xp, nullptr, nullptr);
        qq[i] = m.q[i] - h;
        m.run(v0, m.k, m.r0, qq, nsteps, xm, nullptr, nullptr);
        double dl = 0.0;
        for (int64_t c = 0; c < 3 * n; ++c)
            dl += (xp[c] - xm[c]) * (2.0 * (m.x0[c] - tg[c]) + xp[c] + xm[c]);
        fd_q[t] = dl / static_cast<double>(n) / (2.0 * h);
    }
    return 0;
}

} // extern "C"
