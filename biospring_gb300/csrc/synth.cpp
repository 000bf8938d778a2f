// synth.cpp -- seeded synthetic-system geometry (host C++, no CUDA).
//
// The workloads are synthetic: compact Calpha-like chains (a confined
// self-avoiding random walk) and uniform particle fillings with a minimum
// separation (random sequential addition). Only +, -, *, / and sqrt are used on
// a splitmix64 stream, and the file is compiled with -ffp-contract=off, so a
// seed gives the same coordinates on x86-64 and aarch64.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

namespace
{

struct Rng
{
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return static_cast<double>(next() >> 11) * (1.0 / 9007199254740992.0); }
};

// Uniform bucket grid over an axis-aligned cube [lo, lo + span)^3.
struct Buckets
{
    double lo, cell;
    int64_t dim;
    std::vector<int64_t> head, next;
    Buckets(double lo_, double span, double cell_, int64_t capacity) : lo(lo_), cell(cell_)
    {
        dim = static_cast<int64_t>(span / cell) + 1;
        if (dim < 1)
            dim = 1;
        head.assign(static_cast<size_t>(dim * dim * dim), -1);
        next.assign(static_cast<size_t>(capacity), -1);
    }
    int64_t coord(double v) const
    {
        int64_t c = static_cast<int64_t>((v - lo) / cell);
        return c < 0 ? 0 : (c >= dim ? dim - 1 : c);
    }
    void insert(int64_t id, const double * p)
    {
        const int64_t c = (coord(p[2]) * dim + coord(p[1])) * dim + coord(p[0]);
        next[id] = head[c];
        head[c] = id;
    }
    // Removes `id`, which must be the latest insertion into its bucket.
    void pop(int64_t id, const double * p)
    {
        const int64_t c = (coord(p[2]) * dim + coord(p[1])) * dim + coord(p[0]);
        if (head[c] == id)
            head[c] = next[id];
    }
    // True if some stored point other than `skip` lies closer than r to p.
    bool any_within(const double * p, double r, const std::vector<double> & pts, int64_t skip) const
    {
        const int64_t cx = coord(p[0]), cy = coord(p[1]), cz = coord(p[2]);
        const int64_t reach = static_cast<int64_t>(std::ceil(r / cell));
        const double r2 = r * r;
        for (int64_t z = cz - reach; z <= cz + reach; ++z)
            for (int64_t y = cy - reach; y <= cy + reach; ++y)
                for (int64_t x = cx - reach; x <= cx + reach; ++x)
                {
                    if (x < 0 || y < 0 || z < 0 || x >= dim || y >= dim || z >= dim)
                        continue;
                    for (int64_t id = head[(z * dim + y) * dim + x]; id >= 0; id = next[id])
                    {
                        if (id == skip)
                            continue;
                        const double dx = pts[3 * id] - p[0], dy = pts[3 * id + 1] - p[1], dz = pts[3 * id + 2] - p[2];
                        if (dx * dx + dy * dy + dz * dz < r2)
                            return true;
                    }
                }
        return false;
    }
};

} // namespace

extern "C" {

// Confined self-avoiding walk of n beads with fixed bond length `step`, kept
// inside a ball whose uniform-filling radius of gyration is rg_target
// (R = sqrt(5/3) * rg_target); non-bonded beads stay >= min_sep apart. When a bead
// cannot be placed in 200 trials the walk steps back 1 to 8 beads; after 4n such
// backtracks the ball grows by 1%. Writes float
// xyz[3n] centred on the origin and returns the radius actually used.
double bs_synth_ca_chain(int64_t n, uint64_t seed, double step, double rg_target, double min_sep, float * xyz)
{
    Rng rng(seed);
    double R = std::sqrt(5.0 / 3.0) * rg_target;
    const double span = 4.0 * R + 8.0 * step;
    Buckets grid(-span / 2, span, min_sep > 1.0 ? min_sep : 1.0, n);
    std::vector<double> pts(static_cast<size_t>(3 * n), 0.0);
    if (n <= 0)
        return R;
    grid.insert(0, &pts[0]);
    int64_t i = 1;
    long long backtracks = 0;
    while (i < n)
    {
        bool placed = false;
        for (int attempt = 0; attempt < 200 && !placed; ++attempt)
        {
            double d[3], len2;
            do
            {
                d[0] = 2.0 * rng.uniform() - 1.0;
                d[1] = 2.0 * rng.uniform() - 1.0;
                d[2] = 2.0 * rng.uniform() - 1.0;
                len2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            } while (len2 > 1.0 || len2 < 1e-6);
            const double s = step / std::sqrt(len2);
            double c[3] = {pts[3 * (i - 1)] + s * d[0], pts[3 * (i - 1) + 1] + s * d[1], pts[3 * (i - 1) + 2] + s * d[2]};
            if (c[0] * c[0] + c[1] * c[1] + c[2] * c[2] > R * R)
                continue;
            if (grid.any_within(c, min_sep, pts, i - 1))
                continue;
            pts[3 * i] = c[0];
            pts[3 * i + 1] = c[1];
            pts[3 * i + 2] = c[2];
            grid.insert(i, c);
            placed = true;
        }
        if (placed)
        {
            ++i;
            continue;
        }
        // The chain end is walled in: step back 1 to 8 beads (the most recent insertions, so
        // each is at the head of its bucket) and grow again. The ball grows by 1% only if
        // backtracking keeps failing.
        const int64_t back = std::min<int64_t>(i - 1, 1 + static_cast<int64_t>(rng.next() % 8));
        for (int64_t k = 0; k < back; ++k)
        {
            --i;
            grid.pop(i, &pts[3 * i]);
        }
        if (++backtracks % (4 * n) == 0)
            R *= 1.01;
    }
    double cx = 0, cy = 0, cz = 0;
    for (int64_t i = 0; i < n; ++i)
    {
        cx += pts[3 * i];
        cy += pts[3 * i + 1];
        cz += pts[3 * i + 2];
    }
    cx /= n;
    cy /= n;
    cz /= n;
    for (int64_t i = 0; i < n; ++i)
    {
        xyz[3 * i] = static_cast<float>(pts[3 * i] - cx);
        xyz[3 * i + 1] = static_cast<float>(pts[3 * i + 1] - cy);
        xyz[3 * i + 2] = static_cast<float>(pts[3 * i + 2] - cz);
    }
    return R;
}

// Random sequential addition of up to n points in [0, L)^3 with a minimum
// separation; gives up after max_trials consecutive rejections. Returns the
// number of points placed (written to xyz[3*placed]).
int64_t bs_synth_rsa(int64_t n, double L, double min_sep, uint64_t seed, int64_t max_trials, float * xyz)
{
    Rng rng(seed);
    Buckets grid(0.0, L, min_sep, n);
    std::vector<double> pts(static_cast<size_t>(3 * n), 0.0);
    int64_t placed = 0, fails = 0;
    while (placed < n && fails < max_trials)
    {
        double c[3] = {L * rng.uniform(), L * rng.uniform(), L * rng.uniform()};
        if (grid.any_within(c, min_sep, pts, -1))
        {
            ++fails;
            continue;
        }
        fails = 0;
        pts[3 * placed] = c[0];
        pts[3 * placed + 1] = c[1];
        pts[3 * placed + 2] = c[2];
        grid.insert(placed, c);
        ++placed;
    }
    for (int64_t i = 0; i < placed; ++i)
        for (int k = 0; k < 3; ++k)
            xyz[3 * i + k] = static_cast<float>(pts[3 * i + k]);
    return placed;
}

// All pairs i < j with (double) distance < cutoff, written as int32 (i, j) sorted by
// i then j. Returns the pair count (only min(count, cap) are written).
int64_t bs_synth_pairs_within(int64_t n, const float * xyz, double cutoff, int32_t * ij, int64_t cap)
{
    if (n <= 0)
        return 0;
    double lo = xyz[0], hi = xyz[0];
    for (int64_t i = 0; i < 3 * n; ++i)
    {
        lo = xyz[i] < lo ? xyz[i] : lo;
        hi = xyz[i] > hi ? xyz[i] : hi;
    }
    std::vector<double> pts(static_cast<size_t>(3 * n));
    for (int64_t i = 0; i < 3 * n; ++i)
        pts[i] = xyz[i];
    Buckets grid(lo - 1.0, hi - lo + 2.0, cutoff, n);
    for (int64_t i = 0; i < n; ++i)
        grid.insert(i, &pts[3 * i]);
    const double r2 = cutoff * cutoff;
    int64_t count = 0;
    std::vector<int32_t> row;
    for (int64_t i = 0; i < n; ++i)
    {
        row.clear();
        const double * p = &pts[3 * i];
        const int64_t cx = grid.coord(p[0]), cy = grid.coord(p[1]), cz = grid.coord(p[2]);
        for (int64_t z = cz - 1; z <= cz + 1; ++z)
            for (int64_t y = cy - 1; y <= cy + 1; ++y)
                for (int64_t x = cx - 1; x <= cx + 1; ++x)
                {
                    if (x < 0 || y < 0 || z < 0 || x >= grid.dim || y >= grid.dim || z >= grid.dim)
                        continue;
                    for (int64_t j = grid.head[(z * grid.dim + y) * grid.dim + x]; j >= 0; j = grid.next[j])
                    {
                        if (j <= i)
                            continue;
                        const double dx = pts[3 * j] - p[0], dy = pts[3 * j + 1] - p[1], dz = pts[3 * j + 2] - p[2];
                        if (dx * dx + dy * dy + dz * dz < r2)
                            row.push_back(static_cast<int32_t>(j));
                    }
                }
        // insertion sort: rows are short
        for (size_t a = 1; a < row.size(); ++a)
        {
            int32_t v = row[a];
            size_t b = a;
            while (b > 0 && row[b - 1] > v)
            {
                row[b] = row[b - 1];
                --b;
            }
            row[b] = v;
        }
        for (int32_t j : row)
        {
            if (count < cap)
            {
                ij[2 * count] = static_cast<int32_t>(i);
                ij[2 * count + 1] = j;
            }
            ++count;
        }
    }
    return count;
}

} // extern "C"
