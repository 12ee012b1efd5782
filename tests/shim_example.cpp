// Reference-style caller of the C++ shim (include/vfem.hpp): the same sequence
// as the reference's src/main.cpp:60-124 (assemble, loads, solve, compliance).
// Compiled (not run) by tests/test_capi.py; run it on a GPU machine by hand.
#include <cstdio>
#include <map>
#include <set>
#include <vector>

#include "vfem.hpp"

int main() {
    const int nx = 8, ny = 4, nz = 4;
    std::vector<int> voxels(nx * ny * nz, 1);
    double Ke[24][24];
    vfem_hex8_stiffness(1.0, 0.3, &Ke[0][0]);
    std::set<uint64_t> fixedNodes;
    std::map<uint64_t, vfem::Vec3<double>> loadedNodes;
    for (int z = 0; z <= nz; ++z)
        for (int y = 0; y <= ny; ++y) {
            fixedNodes.insert((uint64_t)(z * (ny + 1) + y) * (nx + 1));
            loadedNodes[(uint64_t)(z * (ny + 1) + y) * (nx + 1) + nx] = {0.0, 0.0, -1.0 / ((ny + 1) * (nz + 1))};
        }
    auto A = vfem::assembleSystemMatrix(voxels.data(), nx, ny, nz, Ke, fixedNodes, 3, 0);
    std::vector<double> f(A.rows(), 0.0), u;
    vfem::applyBoundaryConditions(f, loadedNodes, fixedNodes);
    vfem_stats st = vfem::solveWithKompute(A, f, u);
    double compliance = 0;
    for (size_t i = 0; i < f.size(); ++i) compliance += f[i] * u[i];
    std::printf("iterations %lld, relative residual %.3e, compliance %.6f\n", (long long)st.iterations,
                st.rel_residual, compliance);
    return 0;
}
