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

// One level of the hierarchy as planned on the host (setup.cpp); its per-node
// data is built on the device (setup_gpu.cu).
struct LevelPlan {
    Grid g;
    int div = 2;         // coarsening factor from the previous level (1 on level 0)
    double scale = 1.0;  // operator multiplier 2^(level+skip)
};

// Host set-up pieces (setup.cpp).
vfem_status prepareKe(const double* KeIn, KeData& out);
vfem_status planLevels(int nx, int ny, int nz, int numLevels, int skip, std::vector<LevelPlan>& out,
                       std::string& err);
// Per-child diagonal of R^T Ke_child R for the div^3 children of a coarse element (div^3 x 24).
void childDiagTable(const double* Ke, int div, std::vector<double>& tab);
void initGrid(Grid& g, int ex, int ey, int ez);
void hex8Stiffness(double E, double nu, double* Ke);

}  // namespace vfem
