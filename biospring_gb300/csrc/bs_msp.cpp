// bs_msp.cpp -- .msp parameter-file reader for bs_config (host C++).
//
// Same format and error rules as the reference reader
// (src/configuration/SafeConfigurationReader.cpp:11-75): one "group.param = value" per line,
// lines starting with '#' and blank lines ignored, unknown and duplicated parameters rejected,
// booleans spelled true/false/1/0/on/off/yes/no (src/utils/string.hpp:150-161). Every group
// and parameter name of the reference is accepted (src/configuration/Setting.hpp); the ones
// the step does not read (trajectories, grids, insertion vector, sampling) are checked for
// syntax and otherwise ignored. A new group "cuda.*" carries the device-path knobs.

#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <set>
#include <sstream>
#include <string>

#include "../../include/biospring_gb300.h"

namespace
{

std::string trim(const std::string &s)
{
    size_t a = 0, b = s.size();
    while (a < b && std::isspace(static_cast<unsigned char>(s[a])))
        ++a;
    while (b > a && std::isspace(static_cast<unsigned char>(s[b - 1])))
        --b;
    return s.substr(a, b - a);
}

std::string lower(std::string s)
{
    for (char &c : s)
        c = static_cast<char>(std::tolower(static_cast<unsigned char>(c)));
    return s;
}

bool parse_bool(const std::string &v, int32_t &out)
{
    const std::string s = lower(v);
    if (s == "true" || s == "1" || s == "on" || s == "yes")
        out = 1;
    else if (s == "false" || s == "0" || s == "off" || s == "no")
        out = 0;
    else
        return false;
    return true;
}

bool parse_double(const std::string &v, double &out)
{
    std::istringstream iss(v);
    double d;
    if ((iss >> d).fail())
        return false;
    out = d;
    return true;
}

bool parse_int(const std::string &v, int32_t &out)
{
    std::istringstream iss(v);
    int d;
    if ((iss >> d).fail())
        return false;
    out = d;
    return true;
}

const std::set<std::string> &known_names()
{
    static const std::set<std::string> names = [] {
        std::set<std::string> n;
        auto add = [&](const char *group, std::initializer_list<const char *> params) {
            for (const char *p : params)
                n.insert(std::string(group) + "." + p);
        };
        add("simulation", {"nbsteps", "timestep", "samplerate", "neighborskin"});
        add("steric", {"enable", "gridscale", "cutoff", "mode"});
        add("spring", {"enable", "scale", "cutoff"});
        add("hydrophobicity", {"enable", "scale", "cutoff"});
        add("coulomb", {"enable", "scale", "cutoff", "dielectric"});
        add("impala", {"enable", "scale"});
        add("insertionvector", {"enable", "vector"});
        add("viscosity", {"enable", "value"});
        add("pdbtrajectory", {"enable", "path", "frequency"});
        add("xtctrajectory", {"enable", "path", "frequency"});
        add("csvsampling", {"enable", "path", "frequency"});
        add("potentialgrid", {"enable", "path", "scale"});
        add("densitygrid", {"enable", "path", "scale"});
        add("probe", {"enable", "enableelectrostatic", "enablesteric", "x", "y", "z", "mass", "epsilon", "radius",
                      "charge"});
        add("rigidbody", {"enable", "enablesampling", "enablemontecarlo", "montecarlo_translation_norm",
                          "montecarlo_rotation_norm", "montecarlo_temperature"});
        add("cuda", {"dielectricmode", "rebuildevery", "listskin", "impalaz0", "impalaalpha", "precisepositions"});
        return n;
    }();
    return names;
}

int perr(char *err, size_t len, const std::string &m)
{
    if (err && len)
        std::snprintf(err, len, "%s", m.c_str());
    return BS_E_ARG;
}

} // namespace

extern "C" int bs_config_parse_msp(const char *text, bs_config *cfg, char *err, size_t err_len)
{
    if (!text || !cfg)
        return perr(err, err_len, "bs_config_parse_msp: null argument");
    std::istringstream in(text);
    std::string line;
    std::set<std::string> seen;
    bs_config c = *cfg;
    for (size_t lineid = 1; std::getline(in, line); ++lineid)
    {
        line = trim(line);
        if (line.empty() || line[0] == '#')
            continue;
        const size_t eq = line.find('=');
        const std::string where = "SafeConfigurationReader: line " + std::to_string(lineid) + ": ";
        if (eq == std::string::npos)
            return perr(err, err_len, where + "syntax error: expects param = value (found \"" + line + "\")");
        const std::string name = trim(line.substr(0, eq));
        const std::string value = trim(line.substr(eq + 1));
        if (name.empty() || value.empty())
            return perr(err, err_len, where + "syntax error: expects param = value (found \"" + line + "\")");
        if (!known_names().count(name))
            return perr(err, err_len, where + "invalid parameter \"" + name + "\"");
        if (!seen.insert(name).second)
            return perr(err, err_len, where + "duplicate parameter error: \"" + name +
                                          "\" has been found multiple times in the parameter file");
        const size_t dot = name.find('.');
        const std::string group = name.substr(0, dot), param = name.substr(dot + 1);
        bool ok = true;
        double d = 0.0;
        int32_t b = 0;
        if (param == "enable" || param == "enableelectrostatic" || param == "enablesteric" ||
            param == "enablesampling" || param == "enablemontecarlo" || name == "cuda.precisepositions")
        {
            ok = parse_bool(value, b);
            if (!ok)
                return perr(err, err_len, "Configuration: " + name + ": cannot assign value '" + value +
                                              "': cannot interpret boolean");
            if (group == "steric")
                c.steric_enable = b;
            else if (group == "spring")
                c.spring_enable = b;
            else if (group == "hydrophobicity")
                c.hydrophobicity_enable = b;
            else if (group == "coulomb")
                c.coulomb_enable = b;
            else if (group == "impala")
                c.impala_enable = b;
            else if (group == "viscosity")
                c.viscosity_enable = b;
            else if (group == "rigidbody" && param == "enable")
                c.rigidbody_enable = b;
            else if (name == "cuda.precisepositions")
                c.precise_positions = b;
            else if (name == "probe.enable")
                c.probe_enable = b;
            else if (name == "probe.enableelectrostatic")
                c.probe_electrostatic = b;
            else if (name == "probe.enablesteric")
                c.probe_steric = b;
            else if (name == "potentialgrid.enable")
                c.potentialgrid_enable = b;
            else if (name == "densitygrid.enable")
                c.densitygrid_enable = b;
        }
        else if (name == "steric.mode")
        {
            if (value == "linear")
                c.steric_mode = BS_STERIC_LINEAR;
            else if (value == "lennard-jones-12-6Amber" || value == "lennard-jones-8-6Amber")
                c.steric_mode = BS_STERIC_LJ_12_6_AMBER; // the old name is translated (Setting.hpp:300-320)
            else if (value == "lennard-jones-8-6Lewitt")
                c.steric_mode = BS_STERIC_LJ_8_6_LEWITT;
            else if (value == "lennard-jones-8-6Zacharias")
                c.steric_mode = BS_STERIC_LJ_8_6_ZACHARIAS;
            else
                return perr(err, err_len, "cannot assign value '" + value + "': invalid choice");
        }
        else if (name == "cuda.dielectricmode")
        {
            if (value == "constant")
                c.dielectric_mode = BS_DIELECTRIC_CONSTANT;
            else if (value == "distance")
                c.dielectric_mode = BS_DIELECTRIC_DISTANCE;
            else
                return perr(err, err_len, "cuda.dielectricmode: expects constant or distance");
        }
        else if (name == "simulation.nbsteps" || name == "cuda.rebuildevery")
        {
            int32_t v = 0;
            if (!parse_int(value, v))
                return perr(err, err_len, name + ": cannot interpret integer '" + value + "'");
            if (name == "simulation.nbsteps")
                c.nbsteps = v;
            else
                c.rebuild_every = v;
        }
        else if (name == "potentialgrid.path" || name == "densitygrid.path")
        {
            char *dst = name[0] == 'p' ? c.potentialgrid_path : c.densitygrid_path;
            if (value.size() >= sizeof(c.potentialgrid_path))
                return perr(err, err_len, name + ": path longer than " +
                                              std::to_string(sizeof(c.potentialgrid_path) - 1) + " characters");
            std::snprintf(dst, sizeof(c.potentialgrid_path), "%s", value.c_str());
        }
        else if (param == "path" || param == "vector")
        {
            // accepted, not read by the step
        }
        else
        {
            if (!parse_double(value, d))
                return perr(err, err_len, name + ": cannot interpret number '" + value + "'");
            if (name == "simulation.timestep")
                c.timestep = d;
            else if (name == "simulation.neighborskin")
                c.neighborskin = d;
            else if (name == "steric.gridscale")
                c.steric_gridscale = d;
            else if (name == "steric.cutoff")
                c.steric_cutoff = d;
            else if (name == "spring.scale")
                c.spring_scale = d;
            else if (name == "hydrophobicity.scale")
                c.hydrophobicity_scale = d;
            else if (name == "hydrophobicity.cutoff")
                c.hydrophobicity_cutoff = d;
            else if (name == "coulomb.scale")
                c.coulomb_scale = d;
            else if (name == "coulomb.cutoff")
                c.coulomb_cutoff = d;
            else if (name == "coulomb.dielectric")
                c.coulomb_dielectric = d;
            else if (name == "impala.scale")
                c.impala_scale = d;
            else if (name == "viscosity.value")
                c.viscosity_value = d;
            else if (name == "cuda.listskin")
                c.list_skin = d;
            else if (name == "cuda.impalaz0")
                c.impala_z0 = d;
            else if (name == "cuda.impalaalpha")
                c.impala_alpha = d;
            else if (name == "probe.x")
                c.probe_x = d;
            else if (name == "probe.y")
                c.probe_y = d;
            else if (name == "probe.z")
                c.probe_z = d;
            else if (name == "probe.mass")
                c.probe_mass = d;
            else if (name == "probe.epsilon")
                c.probe_epsilon = d;
            else if (name == "probe.radius")
                c.probe_radius = d;
            else if (name == "probe.charge")
                c.probe_charge = d;
            else if (name == "potentialgrid.scale")
                c.potentialgrid_scale = d;
            else if (name == "densitygrid.scale")
                c.densitygrid_scale = d;
        }
    }
    *cfg = c;
    return BS_OK;
}
