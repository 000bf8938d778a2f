// bs_xtc.cpp -- XTC trajectory frames: GROMACS's compressed coordinate format, which the
// reference writes through its vendored xdrfile library (src/IO/modern/XTCTrajectoryWriter.cpp:
// 15-32: coordinates in nm, identity box, frame counter as step and time, precision 1000).
// Host code only.
//
// The format, as published with GROMACS and the xdrfile library, restated here:
//  * a frame is a sequence of XDR items (big-endian 32-bit words): magic 1995, the atom count,
//    the step, the time (float), the 3 x 3 box (floats), the atom count again; up to 9 atoms
//    follow as plain floats, larger frames as a compressed block: precision (float), the
//    minimum and maximum quantised coordinate per axis (ints), the initial small-delta scale
//    index (int), the block's byte count (int) and the bytes, zero-padded to 4;
//  * coordinates are quantised to integers q = round(x * precision) (halves away from zero);
//  * the block is a bit stream written most significant bit first. Atoms are coded in groups:
//    one atom with its full offset from the minimum corner (three fields of fixed width, or one
//    mixed-radix number when every axis range is below 2^24), then a run of up to 8 following
//    atoms whose per-axis steps from their predecessor are all below half the current scale,
//    each as one mixed-radix number of its three offset steps. A 1-bit flag says whether the
//    run length changed (then 5 bits give run * 3 + scale change + 1). When the first atom
//    after the full one is close, the two are swapped (a water molecule's oxygen then sits next
//    to its hydrogens), and a reader swaps them back;
//  * the scale follows a fixed table of about 2^(k/3), so three values below entry k fit in k
//    bits; it moves one entry up after a group whose full atom was within half the scale limit of
//    the previous atom, and one entry down when a group's steps were all within half the entry
//    below, bounded to eight entries above the start.
// The table and these rules are the format's: a reader decodes exactly what they describe.

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <climits>
#include <vector>

#include "../../include/biospring_gb300.h"

namespace
{

// The format's scale table: entry k ~ 2^(k/3); entries below 9 are unused.
constexpr int kScale[] = {0,       0,       0,       0,       0,       0,       0,       0,       0,       8,
                          10,      12,      16,      20,      25,      32,      40,      50,      64,      80,
                          101,     128,     161,     203,     256,     322,     406,     512,     645,     812,
                          1024,    1290,    1625,    2048,    2580,    3250,    4096,    5060,    6501,    8192,
                          10321,   13003,   16384,   20642,   26007,   32768,   41285,   52015,   65536,   82570,
                          104031,  131072,  165140,  208063,  262144,  330280,  416127,  524287,  660561,  832255,
                          1048576, 1321122, 1664510, 2097152, 2642245, 3329021, 4194304, 5284491, 6658042, 8388607,
                          10568983, 13316085, 16777216};
constexpr int kScaleFirst = 9;
constexpr int kScaleEnd = static_cast<int>(sizeof(kScale) / sizeof(kScale[0])); // one past the last entry
constexpr int kMagic = 1995;
constexpr int kMaxRunInts = 8 * 3;
constexpr double kMaxAbs = static_cast<double>(INT_MAX - 2);

// Entry k, the last one for k past the table (the start index is one past the table when every
// step between consecutive atoms exceeds the largest entry).
int scale_at(int k) { return kScale[k < kScaleEnd ? k : kScaleEnd - 1]; }

// Number of bits of v (0 for 0), at most 32.
int bit_length(unsigned long long v)
{
    int b = 0;
    while (v != 0 && b < 64)
    {
        ++b;
        v >>= 1;
    }
    return b;
}

// Bits the format reserves for a triple of offsets below s0, s1, s2: the bit length of the
// product s0 s1 s2 (one more than strictly needed when the product is a power of two).
int triple_bits(const int s[3])
{
    const unsigned __int128 p = static_cast<unsigned __int128>(static_cast<unsigned>(s[0])) *
                                static_cast<unsigned>(s[1]) * static_cast<unsigned>(s[2]);
    const unsigned long long hi = static_cast<unsigned long long>(p >> 64);
    return hi ? 64 + bit_length(hi) : bit_length(static_cast<unsigned long long>(p));
}

class BitWriter
{
  public:
    // Appends the low `nbits` bits of v, most significant first (any nbits >= 0).
    void put(int nbits, unsigned long long v)
    {
        while (nbits > 32)
        {
            nbits -= 32;
            put32(32, static_cast<uint32_t>(v >> nbits));
        }
        put32(nbits, static_cast<uint32_t>(v));
    }
    std::vector<uint8_t> finish()
    {
        if (nacc_ > 0)
            out_.push_back(static_cast<uint8_t>(acc_ << (8 - nacc_)));
        nacc_ = 0;
        return std::move(out_);
    }

  private:
    void put32(int nbits, uint32_t v)
    {
        if (nbits <= 0)
            return;
        const uint64_t mask = nbits >= 32 ? 0xffffffffull : ((1ull << nbits) - 1ull);
        acc_ = (acc_ << nbits) | (v & mask);
        nacc_ += nbits;
        while (nacc_ >= 8)
        {
            nacc_ -= 8;
            out_.push_back(static_cast<uint8_t>(acc_ >> nacc_));
        }
        acc_ &= (1ull << nacc_) - 1ull;
    }
    std::vector<uint8_t> out_;
    uint64_t acc_ = 0;
    int nacc_ = 0;
};

class BitReader
{
  public:
    BitReader(const uint8_t *p, size_t n) : p_(p), n_(n) {}
    bool get(int nbits, unsigned long long &v)
    {
        v = 0;
        for (int k = 0; k < nbits; ++k)
        {
            if (pos_ >= 8 * n_)
                return false;
            const int bit = (p_[pos_ >> 3] >> (7 - (pos_ & 7))) & 1;
            v = (v << 1) | static_cast<unsigned>(bit);
            ++pos_;
        }
        return true;
    }

  private:
    const uint8_t *p_;
    size_t n_;
    size_t pos_ = 0;
};

// A triple (v0 < s0, v1 < s1, v2 < s2) as the mixed-radix number (v0 s1 + v1) s2 + v2, sent as
// its little-endian bytes in `nbits` bits: whole bytes first, the top byte with the bits left,
// or zero bits after the last byte when the number is shorter than the field.
void put_triple(BitWriter &w, int nbits, const int s[3], const int v[3])
{
    unsigned __int128 x = static_cast<unsigned __int128>(static_cast<unsigned>(v[0])) * static_cast<unsigned>(s[1]) +
                          static_cast<unsigned>(v[1]);
    x = x * static_cast<unsigned>(s[2]) + static_cast<unsigned>(v[2]);
    uint8_t bytes[16];
    int nb = 0;
    do
    {
        bytes[nb++] = static_cast<uint8_t>(x & 0xff);
        x >>= 8;
    } while (x != 0);
    if (nbits >= 8 * nb)
    {
        for (int k = 0; k < nb; ++k)
            w.put(8, bytes[k]);
        w.put(nbits - 8 * nb, 0);
    }
    else
    {
        for (int k = 0; k < nb - 1; ++k)
            w.put(8, bytes[k]);
        w.put(nbits - 8 * (nb - 1), bytes[nb - 1]);
    }
}

bool get_triple(BitReader &r, int nbits, const int s[3], int v[3])
{
    unsigned __int128 x = 0;
    int shift = 0;
    while (nbits > 0)
    {
        const int take = nbits > 8 ? 8 : nbits;
        unsigned long long b;
        if (!r.get(take, b))
            return false;
        x |= static_cast<unsigned __int128>(b) << shift;
        shift += 8;
        nbits -= take;
    }
    v[2] = static_cast<int>(x % static_cast<unsigned>(s[2]));
    x /= static_cast<unsigned>(s[2]);
    v[1] = static_cast<int>(x % static_cast<unsigned>(s[1]));
    x /= static_cast<unsigned>(s[1]);
    v[0] = static_cast<int>(x);
    return true;
}

struct XdrOut
{
    std::vector<uint8_t> b;
    void i32(int32_t v)
    {
        const uint32_t u = static_cast<uint32_t>(v);
        for (int k = 3; k >= 0; --k)
            b.push_back(static_cast<uint8_t>(u >> (8 * k)));
    }
    void f32(float f)
    {
        int32_t v;
        std::memcpy(&v, &f, 4);
        i32(v);
    }
};

struct XdrIn
{
    const uint8_t *p;
    size_t n, at = 0;
    bool i32(int32_t &v)
    {
        if (at + 4 > n)
            return false;
        const uint32_t u = (static_cast<uint32_t>(p[at]) << 24) | (static_cast<uint32_t>(p[at + 1]) << 16) |
                           (static_cast<uint32_t>(p[at + 2]) << 8) | p[at + 3];
        v = static_cast<int32_t>(u);
        at += 4;
        return true;
    }
    bool f32(float &f)
    {
        int32_t v;
        if (!i32(v))
            return false;
        std::memcpy(&f, &v, 4);
        return true;
    }
};

bool within(const int *a, const int *b, int lim)
{
    return std::abs(a[0] - b[0]) < lim && std::abs(a[1] - b[1]) < lim && std::abs(a[2] - b[2]) < lim;
}

// The compressed coordinate block of natoms > 9 atoms; returns BS_OK or BS_E_ARG.
int encode_block(int64_t natoms, const float *xyz, float precision, XdrOut &out)
{
    const size_t n3 = static_cast<size_t>(3 * natoms);
    std::vector<int> q(n3);
    int lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {INT_MIN, INT_MIN, INT_MIN};
    long long min_step = LLONG_MAX;
    for (int64_t i = 0; i < natoms; ++i)
    {
        for (int a = 0; a < 3; ++a)
        {
            float f = xyz[3 * i + a] * precision;
            f = f >= 0.0f ? f + 0.5f : f - 0.5f;
            if (!(std::fabs(static_cast<double>(f)) <= kMaxAbs))
                return BS_E_ARG;
            const int v = static_cast<int>(f);
            q[3 * i + a] = v;
            lo[a] = v < lo[a] ? v : lo[a];
            hi[a] = v > hi[a] ? v : hi[a];
        }
        if (i > 0)
        {
            const long long d = std::llabs(static_cast<long long>(q[3 * i]) - q[3 * i - 3]) +
                                std::llabs(static_cast<long long>(q[3 * i + 1]) - q[3 * i - 2]) +
                                std::llabs(static_cast<long long>(q[3 * i + 2]) - q[3 * i - 1]);
            min_step = d < min_step ? d : min_step;
        }
    }
    out.f32(precision);
    for (int a = 0; a < 3; ++a)
        out.i32(lo[a]);
    for (int a = 0; a < 3; ++a)
        out.i32(hi[a]);
    int range[3];
    for (int a = 0; a < 3; ++a)
    {
        if (static_cast<double>(hi[a]) - static_cast<double>(lo[a]) >= kMaxAbs)
            return BS_E_ARG;
        range[a] = hi[a] - lo[a] + 1;
    }
    const bool wide = range[0] > 0xffffff || range[1] > 0xffffff || range[2] > 0xffffff;
    int field[3] = {0, 0, 0};
    int full_bits = 0;
    if (wide)
        for (int a = 0; a < 3; ++a)
            field[a] = bit_length(static_cast<unsigned>(range[a]));
    else
        full_bits = triple_bits(range);

    int idx = kScaleFirst;
    while (idx < kScaleEnd && scale_at(idx) < min_step)
        ++idx;
    out.i32(idx);
    const int top = idx + 8 < kScaleEnd ? idx + 8 : kScaleEnd;
    const int bottom = top - 8;
    const int up_limit = scale_at(top) / 2;
    int half = scale_at(idx) / 2;                                                   // half the scale
    int half_below = scale_at(idx - 1 > kScaleFirst ? idx - 1 : kScaleFirst) / 2;   // half the entry below
    int sizes[3] = {scale_at(idx), scale_at(idx), scale_at(idx)};

    BitWriter w;
    int prev[3] = {0, 0, 0};
    int last_run = -1; // no run sent yet: the first group always states its run length
    int64_t i = 0;
    while (i < natoms)
    {
        int *cur = &q[3 * i];
        int change;
        if (idx < top && i >= 1 && within(cur, prev, up_limit))
            change = 1;
        else if (idx > bottom)
            change = -1;
        else
            change = 0;
        bool next_close = false;
        if (i + 1 < natoms && within(cur, cur + 3, half))
        {
            for (int a = 0; a < 3; ++a)
                std::swap(cur[a], cur[a + 3]);
            next_close = true;
        }
        const int off[3] = {cur[0] - lo[0], cur[1] - lo[1], cur[2] - lo[2]};
        if (wide)
            for (int a = 0; a < 3; ++a)
                w.put(field[a], static_cast<unsigned>(off[a]));
        else
            put_triple(w, full_bits, range, off);
        std::memcpy(prev, cur, sizeof prev);
        ++i;
        if (!next_close && change == -1)
            change = 0;
        int steps[kMaxRunInts];
        int run = 0;
        while (next_close && run < kMaxRunInts)
        {
            cur = &q[3 * i];
            if (change == -1)
            {
                const long long dx = cur[0] - prev[0], dy = cur[1] - prev[1], dz = cur[2] - prev[2];
                if (dx * dx + dy * dy + dz * dz >= static_cast<long long>(half_below) * half_below)
                    change = 0;
            }
            for (int a = 0; a < 3; ++a)
                steps[run + a] = cur[a] - prev[a] + half;
            run += 3;
            std::memcpy(prev, cur, sizeof prev);
            ++i;
            next_close = i < natoms && within(&q[3 * i], prev, half);
        }
        if (run != last_run || change != 0)
        {
            last_run = run;
            w.put(1, 1);
            w.put(5, static_cast<unsigned>(run + change + 1));
        }
        else
            w.put(1, 0);
        for (int k = 0; k < run; k += 3)
            put_triple(w, idx, sizes, steps + k);
        if (change != 0)
        {
            idx += change;
            if (change < 0)
            {
                half = half_below;
                half_below = idx > kScaleFirst ? scale_at(idx - 1) / 2 : 0;
            }
            else
            {
                half_below = half;
                half = scale_at(idx) / 2;
            }
            sizes[0] = sizes[1] = sizes[2] = scale_at(idx);
        }
    }
    const std::vector<uint8_t> bits = w.finish();
    out.i32(static_cast<int32_t>(bits.size()));
    out.b.insert(out.b.end(), bits.begin(), bits.end());
    while (out.b.size() % 4)
        out.b.push_back(0);
    return BS_OK;
}

int decode_block(XdrIn &in, int64_t natoms, float *xyz, float *precision)
{
    float prec;
    int32_t lo[3], hi[3], idx, nbytes;
    if (!in.f32(prec))
        return BS_E_ARG;
    for (int a = 0; a < 3; ++a)
        if (!in.i32(lo[a]))
            return BS_E_ARG;
    for (int a = 0; a < 3; ++a)
        if (!in.i32(hi[a]))
            return BS_E_ARG;
    if (!in.i32(idx) || !in.i32(nbytes) || idx < kScaleFirst || idx > kScaleEnd || nbytes < 0 ||
        in.at + static_cast<size_t>(nbytes) > in.n || !(prec > 0.0f))
        return BS_E_ARG;
    if (precision)
        *precision = prec;
    int range[3];
    for (int a = 0; a < 3; ++a)
    {
        if (hi[a] < lo[a])
            return BS_E_ARG;
        range[a] = static_cast<int>(static_cast<long long>(hi[a]) - lo[a] + 1);
    }
    const bool wide = range[0] > 0xffffff || range[1] > 0xffffff || range[2] > 0xffffff;
    int field[3] = {0, 0, 0};
    int full_bits = 0;
    if (wide)
        for (int a = 0; a < 3; ++a)
            field[a] = bit_length(static_cast<unsigned>(range[a]));
    else
        full_bits = triple_bits(range);
    int half = scale_at(idx) / 2;
    int half_below = scale_at(idx - 1 > kScaleFirst ? idx - 1 : kScaleFirst) / 2;
    int sizes[3] = {scale_at(idx), scale_at(idx), scale_at(idx)};
    BitReader r(in.p + in.at, static_cast<size_t>(nbytes));
    const float inv = 1.0f / prec;
    int run = 0;
    int64_t i = 0;
    auto emit = [&](int64_t k, const int c[3]) {
        xyz[3 * k] = static_cast<float>(c[0]) * inv;
        xyz[3 * k + 1] = static_cast<float>(c[1]) * inv;
        xyz[3 * k + 2] = static_cast<float>(c[2]) * inv;
    };
    while (i < natoms)
    {
        int full[3];
        if (wide)
        {
            for (int a = 0; a < 3; ++a)
            {
                unsigned long long v;
                if (!r.get(field[a], v))
                    return BS_E_ARG;
                full[a] = static_cast<int>(v);
            }
        }
        else if (!get_triple(r, full_bits, range, full))
            return BS_E_ARG;
        for (int a = 0; a < 3; ++a)
            full[a] += lo[a];
        unsigned long long flag;
        if (!r.get(1, flag))
            return BS_E_ARG;
        int change = 0;
        if (flag)
        {
            unsigned long long code;
            if (!r.get(5, code))
                return BS_E_ARG;
            const int c = static_cast<int>(code);
            change = c % 3;
            run = c - change;
            change -= 1;
        }
        if (i + 1 + run / 3 > natoms)
            return BS_E_ARG;
        if (run == 0)
            emit(i++, full);
        int prev[3] = {full[0], full[1], full[2]};
        for (int k = 0; k < run; k += 3)
        {
            int st[3];
            if (!get_triple(r, idx, sizes, st))
                return BS_E_ARG;
            int c[3] = {prev[0] + st[0] - half, prev[1] + st[1] - half, prev[2] + st[2] - half};
            if (k == 0)
            {
                // the writer swapped the first two atoms of the group: undo it
                emit(i++, c);
                emit(i++, full);
            }
            else
                emit(i++, c);
            std::memcpy(prev, c, sizeof prev); // the next step is from this atom (the first one after a swap)
        }
        idx += change;
        if (idx < kScaleFirst || idx > kScaleEnd)
            return BS_E_ARG;
        if (change < 0)
        {
            half = half_below;
            half_below = idx > kScaleFirst ? scale_at(idx - 1) / 2 : 0;
        }
        else if (change > 0)
        {
            half_below = half;
            half = scale_at(idx) / 2;
        }
        sizes[0] = sizes[1] = sizes[2] = scale_at(idx);
    }
    in.at += (static_cast<size_t>(nbytes) + 3) / 4 * 4;
    return in.at <= in.n ? BS_OK : BS_E_ARG;
}

} // namespace

extern "C" {

int bs_xtc_frame_bound(int64_t natoms, size_t *bytes)
{
    if (!bytes || natoms < 0)
        return BS_E_ARG;
    *bytes = 128 + static_cast<size_t>(natoms) * 16;
    return BS_OK;
}

int bs_xtc_encode_frame(int64_t natoms, int32_t step, float time, const float box[9], const float *xyz,
                        float precision, uint8_t *out, size_t cap, size_t *len)
{
    if (natoms < 0 || natoms > (1ll << 30) || (natoms > 0 && !xyz) || !out || !len || !(precision > 0.0f))
        return BS_E_ARG;
    XdrOut o;
    o.b.reserve(128 + static_cast<size_t>(natoms) * 8);
    o.i32(kMagic);
    o.i32(static_cast<int32_t>(natoms));
    o.i32(step);
    o.f32(time);
    for (int k = 0; k < 9; ++k)
        o.f32(box ? box[k] : (k % 4 == 0 ? 1.0f : 0.0f));
    o.i32(static_cast<int32_t>(natoms));
    if (natoms <= 9)
    {
        for (int64_t k = 0; k < 3 * natoms; ++k)
            o.f32(xyz[k]);
    }
    else
    {
        const int rc = encode_block(natoms, xyz, precision, o);
        if (rc != BS_OK)
            return rc;
    }
    *len = o.b.size();
    if (o.b.size() > cap)
        return BS_E_CAPACITY;
    std::memcpy(out, o.b.data(), o.b.size());
    return BS_OK;
}

int bs_xtc_decode_frame(const uint8_t *in, size_t len, int64_t natoms, int32_t *step, float *time, float box[9],
                        float *xyz, float *precision, size_t *consumed)
{
    if (!in || !xyz || natoms < 0)
        return BS_E_ARG;
    XdrIn r{in, len};
    int32_t magic, n1, st, n2;
    float t;
    float b[9];
    if (!r.i32(magic) || magic != kMagic || !r.i32(n1) || !r.i32(st) || !r.f32(t))
        return BS_E_ARG;
    for (int k = 0; k < 9; ++k)
        if (!r.f32(b[k]))
            return BS_E_ARG;
    if (!r.i32(n2) || n1 != n2 || n1 != natoms)
        return BS_E_ARG;
    if (natoms <= 9)
    {
        for (int64_t k = 0; k < 3 * natoms; ++k)
            if (!r.f32(xyz[k]))
                return BS_E_ARG;
        if (precision)
            *precision = 0.0f;
    }
    else
    {
        const int rc = decode_block(r, natoms, xyz, precision);
        if (rc != BS_OK)
            return rc;
    }
    if (step)
        *step = st;
    if (time)
        *time = t;
    if (box)
        std::memcpy(box, b, sizeof b);
    if (consumed)
        *consumed = r.at;
    return BS_OK;
}

} // extern "C"
