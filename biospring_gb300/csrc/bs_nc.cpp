// bs_nc.cpp -- BioSpring topologies from NetCDF classic files (CDF-1, CDF-2 and CDF-5), without
// the NetCDF library: a reader of the published classic file format (big-endian header of
// dimensions, attributes and variables, then each variable's values at its offset) that returns
// the variables BioSpring's NetCDFReader reads (src/IO/NetCDFReader.cpp:67-203), with its checks.

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>
#include <string>
#include <vector>

#include "../../include/biospring_gb300.h"
#include "bs_nc.h"

namespace bsg
{

namespace
{

enum NcType
{
    NC_BYTE = 1,
    NC_CHAR = 2,
    NC_SHORT = 3,
    NC_INT = 4,
    NC_FLOAT = 5,
    NC_DOUBLE = 6,
    NC_UBYTE = 7,
    NC_USHORT = 8,
    NC_UINT = 9,
    NC_INT64 = 10,
    NC_UINT64 = 11,
};

int type_size(int t)
{
    switch (t)
    {
    case NC_BYTE:
    case NC_CHAR:
    case NC_UBYTE:
        return 1;
    case NC_SHORT:
    case NC_USHORT:
        return 2;
    case NC_INT:
    case NC_FLOAT:
    case NC_UINT:
        return 4;
    case NC_DOUBLE:
    case NC_INT64:
    case NC_UINT64:
        return 8;
    default:
        return 0;
    }
}

struct Var
{
    std::string name;
    std::vector<int> dims;
    int type = 0;
    uint64_t begin = 0;
    uint64_t vsize = 0;
};

struct Header
{
    int version = 0;
    uint64_t numrecs = 0;
    std::vector<std::string> dim_names;
    std::vector<uint64_t> dim_len; // 0 for the record dimension
    int record_dim = -1;
    std::vector<Var> vars;
};

class Cursor
{
  public:
    explicit Cursor(const std::vector<unsigned char> &b) : b_(b) {}
    bool ok() const { return ok_; }
    uint64_t u(int bytes)
    {
        if (pos_ + bytes > b_.size())
        {
            ok_ = false;
            return 0;
        }
        uint64_t v = 0;
        for (int k = 0; k < bytes; ++k)
            v = (v << 8) | b_[pos_ + k];
        pos_ += bytes;
        return v;
    }
    std::string name(int count_bytes)
    {
        const uint64_t n = u(count_bytes);
        if (!ok_ || pos_ + n > b_.size())
        {
            ok_ = false;
            return {};
        }
        std::string s(reinterpret_cast<const char *>(b_.data() + pos_), n);
        pos_ += (n + 3) / 4 * 4;
        return s;
    }
    void skip(uint64_t n)
    {
        if (pos_ + n > b_.size())
            ok_ = false;
        else
            pos_ += n;
    }

  private:
    const std::vector<unsigned char> &b_;
    size_t pos_ = 0;
    bool ok_ = true;
};

bool parse_header(const std::vector<unsigned char> &buf, Header &h, std::string &err)
{
    if (buf.size() < 4 || buf[0] != 'C' || buf[1] != 'D' || buf[2] != 'F' || (buf[3] != 1 && buf[3] != 2 && buf[3] != 5))
    {
        err = "not a NetCDF classic file (CDF-1, CDF-2 or CDF-5); NetCDF-4/HDF5 files are not read";
        return false;
    }
    h.version = buf[3];
    const int nbytes = h.version == 5 ? 8 : 4;  // NON_NEG and nelems
    const int obytes = h.version == 1 ? 4 : 8;  // OFFSET
    Cursor c(buf);
    c.skip(4);
    h.numrecs = c.u(nbytes);
    // dimensions
    uint64_t tag = c.u(4), n = c.u(nbytes);
    if (tag != 0 && tag != 0x0A)
    {
        err = "malformed dimension list";
        return false;
    }
    for (uint64_t d = 0; d < n && c.ok(); ++d)
    {
        h.dim_names.push_back(c.name(nbytes));
        h.dim_len.push_back(c.u(nbytes));
        if (h.dim_len.back() == 0)
            h.record_dim = static_cast<int>(d);
    }
    // global attributes (skipped)
    auto skip_atts = [&]() {
        const uint64_t t = c.u(4), na = c.u(nbytes);
        if (t != 0 && t != 0x0C)
            return false;
        for (uint64_t a = 0; a < na && c.ok(); ++a)
        {
            c.name(nbytes);
            const int type = static_cast<int>(c.u(4));
            const uint64_t nv = c.u(nbytes);
            const int ts = type_size(type);
            if (!ts)
                return false;
            c.skip((nv * ts + 3) / 4 * 4);
        }
        return c.ok();
    };
    if (!skip_atts())
    {
        err = "malformed attribute list";
        return false;
    }
    tag = c.u(4);
    n = c.u(nbytes);
    if (tag != 0 && tag != 0x0B)
    {
        err = "malformed variable list";
        return false;
    }
    for (uint64_t v = 0; v < n && c.ok(); ++v)
    {
        Var var;
        var.name = c.name(nbytes);
        const uint64_t nd = c.u(nbytes);
        for (uint64_t k = 0; k < nd && c.ok(); ++k)
        {
            const uint64_t id = c.u(nbytes);
            if (id >= h.dim_len.size())
            {
                err = "variable \"" + var.name + "\" refers to an unknown dimension";
                return false;
            }
            var.dims.push_back(static_cast<int>(id));
        }
        if (!skip_atts())
        {
            err = "malformed attribute list of \"" + var.name + "\"";
            return false;
        }
        var.type = static_cast<int>(c.u(4));
        var.vsize = c.u(nbytes);
        var.begin = c.u(obytes);
        if (!type_size(var.type))
        {
            err = "variable \"" + var.name + "\" has an unknown type";
            return false;
        }
        h.vars.push_back(var);
    }
    if (!c.ok())
    {
        err = "truncated header";
        return false;
    }
    return true;
}

template <typename T> T decode(const unsigned char *p, int type)
{
    uint64_t v = 0;
    const int ts = type_size(type);
    for (int k = 0; k < ts; ++k)
        v = (v << 8) | p[k];
    switch (type)
    {
    case NC_BYTE:
        return static_cast<T>(static_cast<int8_t>(v));
    case NC_CHAR:
    case NC_UBYTE:
        return static_cast<T>(static_cast<uint8_t>(v));
    case NC_SHORT:
        return static_cast<T>(static_cast<int16_t>(v));
    case NC_USHORT:
        return static_cast<T>(static_cast<uint16_t>(v));
    case NC_INT:
        return static_cast<T>(static_cast<int32_t>(v));
    case NC_UINT:
        return static_cast<T>(static_cast<uint32_t>(v));
    case NC_INT64:
        return static_cast<T>(static_cast<int64_t>(v));
    case NC_UINT64:
        return static_cast<T>(v);
    case NC_FLOAT:
    {
        const uint32_t w = static_cast<uint32_t>(v);
        float f;
        std::memcpy(&f, &w, 4);
        return static_cast<T>(f);
    }
    default:
    {
        double d;
        std::memcpy(&d, &v, 8);
        return static_cast<T>(d);
    }
    }
}

class NcReader
{
  public:
    bool open(const char *path, std::string &err)
    {
        std::ifstream in(path, std::ios::binary);
        if (!in)
        {
            err = std::string(path) + " not found.";
            return false;
        }
        buf_.assign(std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>());
        return parse_header(buf_, h_, err);
    }

    // the size of a dimension, or -1 when the file has none of that name
    long long dim(const std::string &name) const
    {
        for (size_t d = 0; d < h_.dim_names.size(); ++d)
            if (h_.dim_names[d] == name)
                return static_cast<long long>(static_cast<int>(d) == h_.record_dim ? h_.numrecs : h_.dim_len[d]);
        return -1;
    }

    const Var *var(const std::string &name) const
    {
        for (const Var &v : h_.vars)
            if (v.name == name)
                return &v;
        return nullptr;
    }

    uint64_t dim_size(int id) const { return id == h_.record_dim ? h_.numrecs : h_.dim_len[id]; }

    // NetCDFReader::checkNDims / checkDim (NetCDFReader.cpp:247-264)
    bool check(const Var &v, const std::vector<uint64_t> &shape, std::string &err) const
    {
        if (v.dims.size() != shape.size())
        {
            err = "\"" + v.name + "\" array has " + std::to_string(v.dims.size()) +
                  " dimension(s) whereas it should be " + std::to_string(shape.size()) + ".";
            return false;
        }
        for (size_t k = 0; k < shape.size(); ++k)
            if (dim_size(v.dims[k]) != shape[k])
            {
                err = "Dimension " + std::to_string(k) + " of array \"" + v.name + "\" has size " +
                      std::to_string(dim_size(v.dims[k])) + " whereas it should be " + std::to_string(shape[k]) + ".";
                return false;
            }
        return true;
    }

    // every value of v, converted to T, in row-major order
    template <typename T> bool values(const Var &v, std::vector<T> &out, std::string &err) const
    {
        const int ts = type_size(v.type);
        const bool rec = !v.dims.empty() && v.dims[0] == h_.record_dim;
        uint64_t per = 1; // values per record (or in total for a fixed-size variable)
        for (size_t k = rec ? 1 : 0; k < v.dims.size(); ++k)
        {
            const uint64_t d = dim_size(v.dims[k]);
            if (d != 0 && per > UINT64_MAX / d)
            {
                err = "array \"" + v.name + "\" declares more values than can be counted (damaged header)";
                return false;
            }
            per *= d;
        }
        const uint64_t nrec = rec ? h_.numrecs : 1;
        if (per == 0 || nrec == 0)
        {
            out.clear(); // a zero-length dimension: nothing to read
            return true;
        }
        uint64_t recsize = 0;
        if (rec)
        {
            // the record holds every record variable in turn, each padded to 4 bytes, except a
            // lone record variable
            int nrecvars = 0;
            for (const Var &w : h_.vars)
                if (!w.dims.empty() && w.dims[0] == h_.record_dim)
                {
                    ++nrecvars;
                    recsize += w.vsize;
                }
            if (nrecvars == 1)
                recsize = per * ts;
        }
        // the whole extent must lie in the file before anything is allocated: a damaged header
        // can declare any size (the checks are written so that they cannot overflow)
        const uint64_t size = buf_.size();
        const bool fits =
            nrec == 0 ||
            (v.begin <= size && per <= (size - v.begin) / static_cast<uint64_t>(ts) &&
             (nrec == 1 || (recsize > 0 && nrec - 1 <= (size - v.begin) / recsize &&
                            per <= (size - v.begin - (nrec - 1) * recsize) / static_cast<uint64_t>(ts))));
        if (!fits)
        {
            err = "array \"" + v.name + "\" lies past the end of the file";
            return false;
        }
        out.resize(per * nrec);
        for (uint64_t r = 0; r < nrec; ++r)
        {
            const uint64_t at = v.begin + r * recsize;
            if (at + per * ts > buf_.size())
            {
                err = "array \"" + v.name + "\" lies past the end of the file";
                return false;
            }
            for (uint64_t k = 0; k < per; ++k)
                out[r * per + k] = decode<T>(buf_.data() + at + k * ts, v.type);
        }
        return true;
    }

  private:
    std::vector<unsigned char> buf_;
    Header h_;
};

} // namespace

bool read_topology_nc(const char *path, NcTopology &t, std::string &err)
{
    NcReader f;
    if (!f.open(path, err))
        return false;
    // NetCDFReader::readNumberOfParticles / readNumberOfSprings (NetCDFReader.cpp:207-245)
    const long long np = f.dim("particle_number");
    if (np < 0)
    {
        err = "Dimension \"particle_number\" not present in nc file.";
        return false;
    }
    if (np == 0)
    {
        err = "No particle found in topology";
        return false;
    }
    const uint64_t n = static_cast<uint64_t>(np);
    long long ns = f.dim("spring_number");
    if (ns < 0)
        ns = 0; // the reference warns and reads no springs
    auto need = [&](const char *name, bool mandatory, const std::vector<uint64_t> &shape) -> const Var * {
        const Var *v = f.var(name);
        if (!v)
        {
            if (mandatory)
                err = std::string("Array \"") + name + "\" not found in topology file.";
            return nullptr;
        }
        if (!f.check(*v, shape, err))
            return nullptr;
        return v;
    };
    // NetCDFReader::readParticles (NetCDFReader.cpp:86-181): the mandatory arrays, then the optional
    // IMPALA and hydrophobicity ones
    const char *mandatory1[] = {"particleids", "resids", "dynamicstate", "radii", "mass", "epsilon", "charges"};
    for (const char *name : mandatory1)
        if (!need(name, true, {n}))
            return false;
    const uint64_t names[3] = {4, 4, 4}; // PARTICLE_NAME_LENGTH, RESIDUE_NAME_LENGTH, CHAIN_NAME_LENGTH
    if (!need("resnames", true, {n, names[1]}) || !need("particlenames", true, {n, names[0]}) ||
        !need("chainnames", true, {n, names[2]}))
        return false;
    const Var *coords = need("coordinates", true, {n, 3});
    if (!coords)
        return false;
    t.n = static_cast<int64_t>(n);
    std::vector<unsigned char> dyn;
    std::vector<float> mass;
    if (!f.values(*coords, t.xyz, err) || !f.values(*f.var("charges"), t.charge, err) ||
        !f.values(*f.var("radii"), t.radius, err) || !f.values(*f.var("epsilon"), t.epsilon, err) ||
        !f.values(*f.var("mass"), mass, err) || !f.values(*f.var("dynamicstate"), dyn, err))
        return false;
    t.mass.resize(n);
    t.is_static.resize(n);
    for (uint64_t i = 0; i < n; ++i)
    {
        // NetCDFReader::addParticlesToSpn (NetCDFReader.cpp:31-37): a zero mass becomes 1
        t.mass[i] = std::abs(mass[i]) < 1e-6 ? 1.0f : mass[i];
        t.is_static[i] = dyn[i] == 0 ? 1 : 0;
    }
    t.sasa.clear();
    t.transfer.clear();
    t.hydrophobicity.clear();
    if (const Var *v = need("surfaceaccessibility", false, {n}))
    {
        if (!f.values(*v, t.sasa, err))
            return false;
    }
    else if (!err.empty())
        return false;
    if (const Var *v = need("hydrophobicityscale", false, {n}))
    {
        if (!f.values(*v, t.transfer, err))
            return false;
    }
    else if (!err.empty())
        return false;
    if (const Var *v = need("hydrophobicity", false, {n}))
    {
        if (!f.values(*v, t.hydrophobicity, err))
            return false;
    }
    else if (!err.empty())
        return false;
    // NetCDFReader::readSprings (NetCDFReader.cpp:183-205)
    t.ij.clear();
    t.r0.clear();
    t.k.clear();
    if (ns > 0)
    {
        const uint64_t m = static_cast<uint64_t>(ns);
        const Var *sp = need("springs", true, {m, 2});
        const Var *sk = sp ? need("springsstiffness", true, {m}) : nullptr;
        const Var *sr = sk ? need("springsequilibrium", true, {m}) : nullptr;
        if (!sr)
            return false;
        if (!f.values(*sp, t.ij, err) || !f.values(*sk, t.k, err) || !f.values(*sr, t.r0, err))
            return false;
        for (int32_t id : t.ij)
            if (id < 0 || static_cast<uint64_t>(id) >= n)
            {
                err = "a spring refers to a particle index out of range";
                return false;
            }
    }
    return true;
}

} // namespace bsg

extern "C" int bs_read_nc(const char *path, int64_t *n_particles, int64_t *n_springs, float *xyz, float *mass,
                          float *charge, float *radius, float *epsilon, float *sasa, float *transfer,
                          float *hydrophobicity, uint8_t *is_static, int32_t *ij, float *r0, float *k,
                          int32_t *present, char *err, size_t err_len)
{
    bsg::NcTopology t;
    std::string msg;
    if (!path || !n_particles || !n_springs)
        msg = "bs_read_nc: null argument";
    else if (bsg::read_topology_nc(path, t, msg))
    {
        *n_particles = t.n;
        *n_springs = static_cast<int64_t>(t.r0.size());
        auto put = [](float *dst, const std::vector<float> &v) {
            if (dst && !v.empty())
                std::memcpy(dst, v.data(), sizeof(float) * v.size());
        };
        put(xyz, t.xyz);
        put(mass, t.mass);
        put(charge, t.charge);
        put(radius, t.radius);
        put(epsilon, t.epsilon);
        put(sasa, t.sasa);
        put(transfer, t.transfer);
        put(hydrophobicity, t.hydrophobicity);
        put(r0, t.r0);
        put(k, t.k);
        if (is_static)
            std::memcpy(is_static, t.is_static.data(), t.is_static.size());
        if (ij && !t.ij.empty())
            std::memcpy(ij, t.ij.data(), sizeof(int32_t) * t.ij.size());
        if (present)
        {
            present[0] = !t.sasa.empty();
            present[1] = !t.transfer.empty();
            present[2] = !t.hydrophobicity.empty();
        }
        return BS_OK;
    }
    if (err && err_len)
        std::snprintf(err, err_len, "NetCDFReader: %s", msg.c_str());
    return BS_E_ARG;
}
