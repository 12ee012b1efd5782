// vfem_internal.h -- types shared by the host set-up, the kernels and the C ABI.
//
// Device data layout (one "level" = one grid of the multigrid hierarchy):
//   * nodes live on the dense node grid (ex+1) x (ey+1) x (ez+1), x fastest;
//     node (x,y,z) has storage index s = (z*ny + y)*nx + x;
//   * a vector stores 3 values per node, interleaved: v[3*s + c] (the
//     reference's DOF = 3*node + c, with the compressed node replaced by s);
//     unused nodes hold 0 in every vector;
//   * the element (voxel) with lower corner node s stores its Young's-modulus
//     multiplier at E[s] (0 = empty), so the elements touching node s are
//     s - {0,1}*(1, nx, nx*ny);
//   * node flags: bit 0 used, bit 1 fixed.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "vfem.h"

namespace vfem {

enum : uint8_t { FLAG_USED = 1, FLAG_FIXED = 2 };

struct Grid {
    int ex, ey, ez;  // elements per axis
    int nx, ny, nz;  // nodes per axis (= elements + 1)
    int64_t nnode;   // nx*ny*nz
#ifdef __CUDACC__
    __host__ __device__
#endif
    inline int64_t store(int x, int y, int z) const {
        return ((int64_t)z * ny + y) * nx + x;
    }
};

// Element stiffness data derived once per problem.
struct KeData {
    double Ke[576];      // symmetrised from the upper triangle (src/FEM.cpp:200-210)
    double Khat[576];    // H Ke H^T / 64 in the Walsh basis (per component, 8-point Hadamard)
    bool structured;     // Khat has non-zeros only on the 45-entry isotropic-cube pattern
    double ks[45];       // Khat on that pattern, in pattern order
    double diag[24];
};

// The 45-entry pattern of Khat for a reflection- and rotation-symmetric cube
// element: index i = 3*m + c, m = Walsh mode (bit i <-> axis i), c = component.
extern const int kPatRow[45];
extern const int kPatCol[45];

struct HostLevel {
    Grid g;
    int divider = 2;               // coarsening factor from the previous level
    double scale = 1.0;            // operator multiplier 2^(level+skip)
    std::vector<float> E;          // per element (lower-corner storage index), 0 = empty
    std::vector<float> Ev;         // multiplicative-cycle modulus: volume average of the children
                                   // (empty children count as 0); equals E on the finest level
    std::vector<uint8_t> flags;    // per node
    std::vector<double> dinv;      // 3 per node: reference inverse diagonal (Galerkin for partial elements)
    std::vector<double> dinvRedisc;// 3 per node: inverse diagonal of the rediscretised operator
    std::vector<int32_t> nodeStore;// compressed id -> storage index
    std::vector<int64_t> fixedIds; // compressed ids of fixed nodes, sorted
    int64_t nelem = 0;
};

struct Hierarchy {
    std::vector<HostLevel> L;
    int skip = 0;
    // coarsest level
    std::vector<int32_t> coarseFreeDof;   // storage DOF index (3*s + c) of each free coarse DOF
    std::vector<int32_t> coarseFreeNode;  // storage node -> free node id, -1 otherwise
};

// Host set-up (setup.cpp).
vfem_status prepareKe(const double* KeIn, KeData& out);
vfem_status buildHierarchy(const uint8_t* vox, int nx, int ny, int nz, const float* E,
                           const int64_t* fixed, int64_t nfixed, int numLevels, int skip,
                           const KeData& ke, Hierarchy& H, std::string& err);
void hex8Stiffness(double E, double nu, double* Ke);

}  // namespace vfem
