// bs_nc.h -- BioSpring topology from a NetCDF classic file (host side).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace bsg
{

// The arrays NetCDFReader hands to the SpringNetwork (src/IO/NetCDFReader.cpp:8-65), caller order.
// Optional arrays are empty when the file does not hold them.
struct NcTopology
{
    int64_t n = 0;
    std::vector<float> xyz, charge, radius, epsilon, mass, sasa, transfer, hydrophobicity;
    std::vector<uint8_t> is_static;
    std::vector<int32_t> ij; // 2 per spring
    std::vector<float> r0, k;
};

bool read_topology_nc(const char *path, NcTopology &t, std::string &err);

} // namespace bsg
