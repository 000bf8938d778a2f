// bs_field.h -- host helpers of the field grids (OpenDX reader, per-cell force vectors).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/biospring_gb300.h"

namespace bsg
{

namespace fieldunits
{
// Unit constants of the field-gradient scale (src/forcefield/constants.hpp:53, 58-61, 65-66, 70,
// 80-81); the product is evaluated in double and rounded to float, as the reference does.
constexpr double kBoltzmannJPerK = 1.3806504E-23;
constexpr double kMeterToAngstrom = 1.0E10;
constexpr double kNewtonToDaAFs2 = kMeterToAngstrom * (1.0 / 1.66054E-27) * 1.0E-15 * 1.0E-15;
} // namespace fieldunits

void field_shape(const long counts[3], const double origin[3], const double spacing[3], int shape[3]);
bool read_dx(const char *path, int shape[3], double origin[3], double spacing[3], std::vector<float> *values,
             std::string &err);
void field_cells(const int shape[3], const double spacing[3], const float *scalar, float *cells);

} // namespace bsg
