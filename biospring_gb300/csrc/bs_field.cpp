// bs_field.cpp -- host side of the field grids: the OpenDX scalar-map reader and the per-cell
// force vectors, restating the reference's OpenDXReader (src/IO/OpenDXReader.cpp) and
// PotentialGrid::compute_gradient (src/grid/PotentialGrid.cpp:20-59) with the same float and
// double roundings, so that the device looks up the very cell values the reference would.

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "bs_field.h"

namespace bsg
{

namespace
{

std::vector<std::string> words(const std::string &s)
{
    std::vector<std::string> out;
    std::istringstream in(s);
    std::string w;
    while (in >> w)
        out.push_back(w);
    return out;
}

// std::stof / std::stoi semantics: leading number of the token, an error when there is none or it
// is out of range.
bool to_float(const std::string &t, float &v)
{
    errno = 0;
    char *end = nullptr;
    v = std::strtof(t.c_str(), &end);
    return end != t.c_str() && errno != ERANGE;
}

bool to_int(const std::string &t, long &v)
{
    errno = 0;
    char *end = nullptr;
    v = std::strtol(t.c_str(), &end, 10);
    return end != t.c_str() && errno != ERANGE && v >= INT32_MIN && v <= INT32_MAX;
}

bool fail(std::string &err, const std::string &m)
{
    err = "OpenDXReader: " + m;
    return false;
}

} // namespace

// Cells per axis of a grid over the box [origin, origin + counts * spacing], as the reference's
// GridCoordinatesSystem::initialize derives them (ceil(length / cell size), GridCoordinatesSystem.hpp:
// 180-191); normally equal to counts.
void field_shape(const long counts[3], const double origin[3], const double spacing[3], int shape[3])
{
    for (int a = 0; a < 3; ++a)
    {
        const double hi = origin[a] + static_cast<double>(static_cast<size_t>(counts[a])) * spacing[a];
        shape[a] = static_cast<int>(static_cast<size_t>(std::ceil((hi - origin[a]) / spacing[a])));
    }
}

bool read_dx(const char *path, int shape[3], double origin[3], double spacing[3], std::vector<float> *values,
             std::string &err)
{
    std::ifstream in(path);
    if (!in)
        return fail(err, std::string("cannot open '") + path + "'");
    std::ifstream probe(path, std::ios::binary | std::ios::ate);
    const double file_bytes = probe ? static_cast<double>(probe.tellg()) : -1.0;
    std::string line;
    // comment lines, then the grid counts
    do
    {
        if (!std::getline(in, line))
            return fail(err, "cannot read grid dimensions (end of file)");
    } while (line.substr(0, 1) == "#");
    const std::string key = "object 1 class gridpositions counts";
    if (line.size() < key.size() || line.compare(0, key.size(), key) != 0)
        return fail(err, "cannot read grid dimensions (found " + line + ")");
    std::vector<std::string> t = words(line.substr(key.size()));
    long counts[3];
    if (t.size() != 3 || !to_int(t[0], counts[0]) || !to_int(t[1], counts[1]) || !to_int(t[2], counts[2]))
        return fail(err, "cannot read grid dimensions (found '" + line + "')");
    if (!std::getline(in, line) || line.substr(0, 6) != "origin")
        return fail(err, "cannot read grid origin (found '" + line + "')");
    t = words(line.size() > 7 ? line.substr(7) : std::string());
    float o[3];
    if (t.size() != 3 || !to_float(t[0], o[0]) || !to_float(t[1], o[1]) || !to_float(t[2], o[2]))
        return fail(err, "cannot read grid origin (found '" + line + "')");
    float delta[3] = {0.f, 0.f, 0.f};
    for (int r = 0; r < 3; ++r)
    {
        if (!std::getline(in, line) || line.substr(0, 5) != "delta")
            return fail(err, "cannot read scaling factors (found '" + line + "')");
        t = words(line.size() > 6 ? line.substr(6) : std::string());
        float d[3];
        if (t.size() != 3 || !to_float(t[0], d[0]) || !to_float(t[1], d[1]) || !to_float(t[2], d[2]))
            return fail(err, "cannot read scaling factors (found '" + line + "')");
        delta[r] = d[r]; // the diagonal
    }
    // A damaged header may declare anything: the counts, the cell sizes and the number of values
    // the file can hold (at least two characters each) are checked before any size is derived
    // or allocated.
    constexpr long kMaxCount = 1L << 24;
    for (int a = 0; a < 3; ++a)
    {
        if (counts[a] < 0)
            return fail(err, "cannot read grid dimensions (negative count)");
        if (counts[a] > kMaxCount)
            return fail(err, "cannot read grid dimensions (more than 16777216 points along an axis)");
        if (!(delta[a] > 0.0f) || !std::isfinite(delta[a]) || !std::isfinite(o[a]))
            return fail(err, "cannot read scaling factors (a finite cell size > 0 and a finite origin are "
                             "required)");
        origin[a] = static_cast<double>(o[a]);
        spacing[a] = static_cast<double>(delta[a]);
    }
    const double declared = static_cast<double>(counts[0]) * static_cast<double>(counts[1]) *
                            static_cast<double>(counts[2]);
    if (file_bytes >= 0.0 && declared > file_bytes / 2.0 + 1.0)
        return fail(err, "cannot access grid data (the file is too short for the " + std::to_string(counts[0]) +
                             " x " + std::to_string(counts[1]) + " x " + std::to_string(counts[2]) +
                             " values declared)");
    field_shape(counts, origin, spacing, shape);
    if (!values)
        return true;
    // "object 2 class gridconnections ..." and "object 3 class array ... data follows"
    std::getline(in, line);
    std::getline(in, line);
    const size_t total = static_cast<size_t>(shape[0]) * static_cast<size_t>(shape[1]) * static_cast<size_t>(shape[2]);
    values->assign(total, 0.0f);
    size_t count = 0;
    while (count < total)
    {
        if (!std::getline(in, line))
            return fail(err, "cannot access grid data");
        t = words(line);
        if (t.empty() || t.size() > 3)
            return fail(err, "misformatted grid data (expected 1 to 3 tokens, found '" + line + "'");
        for (const std::string &w : t)
        {
            if (count >= total)
                return fail(err, "more grid data than the declared " + std::to_string(total) + " values");
            float v;
            if (!to_float(w, v))
                return fail(err, "misformatted grid value '" + w + "'");
            (*values)[count++] = v * 1.0f;
        }
    }
    return true;
}

// Force vector of every cell from the scalar map: the centred difference along each axis
// (zero on the grid's first and last layer), times -k_B * 1e10 * (N -> Da A fs^-2), as
// PotentialGrid::compute_gradient (PotentialGrid.cpp:20-59): float differences, a double
// division by (float spacing) * 2.0 rounded to float, a float product with the float scale.
void field_cells(const int shape[3], const double spacing[3], const float *scalar, float *cells)
{
    using namespace fieldunits;
    const float scale = static_cast<float>(kBoltzmannJPerK * kMeterToAngstrom * kNewtonToDaAFs2);
    const float h[3] = {static_cast<float>(spacing[0]), static_cast<float>(spacing[1]), static_cast<float>(spacing[2])};
    const size_t n0 = static_cast<size_t>(shape[0]), n1 = static_cast<size_t>(shape[1]),
                 n2 = static_cast<size_t>(shape[2]);
    auto at = [&](size_t i, size_t j, size_t k) { return scalar[(i * n1 + j) * n2 + k]; };
    auto centred = [](float cur, float prev, float next, float hh) {
        return static_cast<float>(static_cast<double>((cur - prev) + (next - cur)) / (static_cast<double>(hh) * 2.0));
    };
    for (size_t i = 0; i < n0; ++i)
        for (size_t j = 0; j < n1; ++j)
            for (size_t k = 0; k < n2; ++k)
            {
                const float c = at(i, j, k);
                float g[3] = {0.0f, 0.0f, 0.0f};
                if (i > 0 && i + 1 < n0)
                    g[0] = centred(c, at(i - 1, j, k), at(i + 1, j, k), h[0]);
                if (j > 0 && j + 1 < n1)
                    g[1] = centred(c, at(i, j - 1, k), at(i, j + 1, k), h[1]);
                if (k > 0 && k + 1 < n2)
                    g[2] = centred(c, at(i, j, k - 1), at(i, j, k + 1), h[2]);
                float *out = cells + 4 * ((i * n1 + j) * n2 + k);
                out[0] = c;
                out[1] = g[0] * -scale;
                out[2] = g[1] * -scale;
                out[3] = g[2] * -scale;
            }
}

} // namespace bsg

extern "C" int bs_read_dx(const char *path, int32_t shape[3], double origin[3], double spacing[3], float *scalar,
                          char *err, size_t err_len)
{
    std::string msg;
    if (!path || !shape || !origin || !spacing)
        msg = "bs_read_dx: null argument";
    else
    {
        int sh[3];
        std::vector<float> v;
        if (bsg::read_dx(path, sh, origin, spacing, scalar ? &v : nullptr, msg))
        {
            for (int a = 0; a < 3; ++a)
                shape[a] = sh[a];
            if (scalar)
                std::memcpy(scalar, v.data(), sizeof(float) * v.size());
            return BS_OK;
        }
    }
    if (err && err_len)
        std::snprintf(err, err_len, "%s", msg.c_str());
    return BS_E_ARG;
}
