// vfem_inout.hpp -- header-only readers and writers for the reference's model
// files, with the reference's names (src/inout.cpp, include/in.hpp:19-34,
// include/out.hpp:18-63), so that a caller of the reference's I/O switches by
// changing the namespace.
//
//   reference (src/inout.cpp)                          here
//   int* loadVoxel(name, sx, sy, sz)       :6-41       vfem::loadVoxel(name, sx, sy, sz) -> std::vector<int>
//   getKe(name, Ke[24][24])                :43-72      vfem::getKe(name, Ke)
//   getBoundaryConditions(name, fixed, loads) :77-128  vfem::getBoundaryConditions(name, fixed, loads)
//   saveVector(u, name)                    :206-225    vfem::saveVector(u, name[, digits])
//
// File formats (the reference's):
//   <name>.dat          "sx sy sz\n", then sz lines, each the sx*sy values of one
//                       z-slice (x fastest), comma-separated; 1 = filled voxel.
//   <name>_Ke0.dat      24 lines of 24 comma-separated numbers; when absent,
//                       data/Ke0.dat is read instead (inout.cpp:51-56).
//   <name>_fixed.dat    count, then one 1-based node id per line.
//   <name>_loading.dat  count, then "id\tfx\tfy\tfz" per line, 1-based ids.
//   <name>_out.csv      one line, comma-separated values.
// Paths are relative to the working directory, as in the reference.
//
// Differences, all on error or output precision only:
//  * a missing or malformed file throws std::runtime_error naming the file and
//    line (the reference throws std::invalid_argument from std::stoi, or reads
//    garbage from a stream that failed to open);
//  * saveVector writes 17 significant digits by default, which round-trips every
//    double exactly; digits = -1 reproduces the reference's std::to_string form
//    (fixed notation, 6 decimals: values below 5e-7 in magnitude print as 0).
#pragma once

#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "vfem.hpp"

namespace vfem {

namespace detail {

inline std::runtime_error ioError(const std::string& path, long line, const std::string& what) {
    return std::runtime_error(path + ":" + std::to_string(line) + ": " + what);
}

inline std::ifstream openIn(const std::string& path) {
    std::ifstream in(path);
    if (!in) throw std::runtime_error(path + ": cannot open");
    return in;
}

inline long long parseInt(const std::string& tok, const std::string& path, long line) {
    const char* s = tok.c_str();
    char* end = nullptr;
    errno = 0;
    long long v = std::strtoll(s, &end, 10);
    while (end && (*end == ' ' || *end == '\r' || *end == '\t')) ++end;
    if (end == s || errno != 0 || (end && *end != '\0')) throw ioError(path, line, "bad integer '" + tok + "'");
    return v;
}

inline double parseReal(const std::string& tok, const std::string& path, long line) {
    const char* s = tok.c_str();
    char* end = nullptr;
    errno = 0;
    double v = std::strtod(s, &end);
    while (end && (*end == ' ' || *end == '\r' || *end == '\t')) ++end;
    const bool overflow = errno == ERANGE && (v == HUGE_VAL || v == -HUGE_VAL);
    if (end == s || overflow || (end && *end != '\0')) throw ioError(path, line, "bad number '" + tok + "'");
    return v;
}

// Split on sep; a trailing empty field (a line ending in the separator) is dropped.
inline std::vector<std::string> split(const std::string& line, char sep) {
    std::vector<std::string> out;
    std::string cur;
    std::istringstream ss(line);
    while (std::getline(ss, cur, sep)) out.push_back(cur);
    while (!out.empty() && out.back().find_first_not_of(" \r\t") == std::string::npos) out.pop_back();
    return out;
}

inline void getlineOrThrow(std::istream& in, std::string& line, const std::string& path, long lineNo) {
    if (!std::getline(in, line)) throw ioError(path, lineNo, "unexpected end of file");
}

inline bool fileExists(const std::string& path) {
    std::ifstream f(path);
    return (bool)f;
}

}  // namespace detail

// Voxel occupancy of <model_name>.dat, x fastest then y then z (inout.cpp:6-41).
inline std::vector<int> loadVoxel(const std::string& model_name, int& sizeX, int& sizeY, int& sizeZ) {
    const std::string path = model_name + ".dat";
    std::ifstream in = detail::openIn(path);
    std::string line;
    detail::getlineOrThrow(in, line, path, 1);
    {
        std::istringstream ss(line);
        if (!(ss >> sizeX >> sizeY >> sizeZ) || sizeX <= 0 || sizeY <= 0 || sizeZ <= 0)
            throw detail::ioError(path, 1, "bad dimensions line '" + line + "'");
    }
    const long long slice = (long long)sizeX * sizeY;
    std::vector<int> model;
    model.reserve((size_t)(slice * sizeZ));
    for (int z = 0; z < sizeZ; ++z) {
        detail::getlineOrThrow(in, line, path, z + 2);
        std::vector<std::string> toks = detail::split(line, ',');
        if ((long long)toks.size() != slice)
            throw detail::ioError(path, z + 2, "expected " + std::to_string(slice) + " values, found " +
                                                   std::to_string(toks.size()));
        for (const std::string& t : toks) model.push_back((int)detail::parseInt(t, path, z + 2));
    }
    return model;
}

// Occupancy as the C ABI takes it: 1 where the value is 1 (FEM.cpp:75), else 0.
inline std::vector<uint8_t> occupancy(const std::vector<int>& model) {
    std::vector<uint8_t> occ(model.size());
    for (size_t i = 0; i < model.size(); ++i) occ[i] = model[i] == 1 ? 1 : 0;
    return occ;
}

// Element stiffness from <model_name>_Ke0.dat, else data/Ke0.dat (inout.cpp:43-72).
template <typename scalar>
inline void getKe(const std::string& model_name, scalar Ke[24][24]) {
    std::string path = model_name + "_Ke0.dat";
    if (!detail::fileExists(path)) path = "data/Ke0.dat";
    std::ifstream in = detail::openIn(path);
    std::string line;
    for (int i = 0; i < 24; ++i) {
        detail::getlineOrThrow(in, line, path, i + 1);
        std::vector<std::string> toks = detail::split(line, ',');
        if (toks.size() != 24) throw detail::ioError(path, i + 1, "expected 24 values");
        for (int j = 0; j < 24; ++j) Ke[i][j] = (scalar)detail::parseReal(toks[j], path, i + 1);
    }
}

// Fixed nodes (0-based, a set) and loads (0-based node -> force; a later line
// for the same node replaces an earlier one) (inout.cpp:77-128).
template <typename scalar>
inline void getBoundaryConditions(const std::string& model_name, std::set<uint64_t>& fixedNodes,
                                  std::map<uint64_t, Vec3<scalar>>& loadedNodes) {
    std::string line;
    {
        const std::string path = model_name + "_fixed.dat";
        std::ifstream in = detail::openIn(path);
        detail::getlineOrThrow(in, line, path, 1);
        long long n = detail::parseInt(line, path, 1);
        if (n < 0) throw detail::ioError(path, 1, "negative count");
        for (long long i = 0; i < n; ++i) {
            detail::getlineOrThrow(in, line, path, (long)i + 2);
            long long id = detail::parseInt(line, path, (long)i + 2);
            if (id < 1) throw detail::ioError(path, (long)i + 2, "node ids are 1-based");
            fixedNodes.insert((uint64_t)(id - 1));
        }
    }
    {
        const std::string path = model_name + "_loading.dat";
        std::ifstream in = detail::openIn(path);
        detail::getlineOrThrow(in, line, path, 1);
        long long n = detail::parseInt(line, path, 1);
        if (n < 0) throw detail::ioError(path, 1, "negative count");
        for (long long i = 0; i < n; ++i) {
            const long ln = (long)i + 2;
            detail::getlineOrThrow(in, line, path, ln);
            std::vector<std::string> toks = detail::split(line, '\t');
            if (toks.size() != 4) throw detail::ioError(path, ln, "expected id<TAB>fx<TAB>fy<TAB>fz");
            long long id = detail::parseInt(toks[0], path, ln);
            if (id < 1) throw detail::ioError(path, ln, "node ids are 1-based");
            loadedNodes[(uint64_t)(id - 1)] = Vec3<scalar>{(scalar)detail::parseReal(toks[1], path, ln),
                                                           (scalar)detail::parseReal(toks[2], path, ln),
                                                           (scalar)detail::parseReal(toks[3], path, ln)};
        }
    }
}

// One number as saveVector writes it: 17 significant digits (exact round trip)
// or, with digits = -1, std::to_string's fixed 6-decimal form (inout.cpp:215-220).
inline std::string formatValue(double v, int digits = 17) {
    char buf[64];
    if (digits < 0)
        std::snprintf(buf, sizeof buf, "%f", v);
    else
        std::snprintf(buf, sizeof buf, "%.*g", digits, v);
    return buf;
}

// <name>_out.csv: the values on one comma-separated line (inout.cpp:206-225).
template <typename T>
inline void saveVector(const std::vector<T>& data, const std::string& name, int digits = 17) {
    const std::string path = name + "_out.csv";
    std::ofstream out(path);
    if (!out) throw std::runtime_error(path + ": cannot open for writing");
    for (size_t j = 0; j < data.size(); ++j) {
        if (j) out << ',';
        out << formatValue((double)data[j], digits);
    }
    out << '\n';
    if (!out) throw std::runtime_error(path + ": write failed");
}

}  // namespace vfem
