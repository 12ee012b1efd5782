// The reference's command-line driver (src/main.cpp:28-127) written against the
// C++ shims include/vfem_inout.hpp and include/vfem.hpp: load the model files,
// assemble, apply the loads, solve on the GPU, print the compliance, save the
// solution.  With --parse-only it stops after reading and prints what it read
// (sizes, counts and sums), which needs no GPU.
//
//   inout_example <model>.dat [-n L] [--skip S] [--digits D] [--parse-only]
#include <cstdio>
#include <cstring>
#include <map>
#include <set>
#include <string>
#include <vector>

#include "vfem_inout.hpp"

int main(int argc, char** argv) {
    if (argc < 2) {
        std::printf("An input file is necessary\n");
        return 1;
    }
    std::string fileName(argv[1]);
    std::string modelName = fileName.substr(0, fileName.find('.', 1));
    int numLevels = 3, skipLevels = 0, digits = 17;
    bool parseOnly = false;
    for (int i = 2; i < argc; ++i) {
        if (!std::strcmp(argv[i], "-n") && i + 1 < argc) numLevels = std::atoi(argv[++i]);
        else if (!std::strcmp(argv[i], "--skip") && i + 1 < argc) skipLevels = std::atoi(argv[++i]);
        else if (!std::strcmp(argv[i], "--digits") && i + 1 < argc) digits = std::atoi(argv[++i]);
        else if (!std::strcmp(argv[i], "--parse-only")) parseOnly = true;
    }
    try {
        int sx, sy, sz;
        std::vector<int> model = vfem::loadVoxel(modelName, sx, sy, sz);
        double Ke[24][24];
        vfem::getKe(modelName, Ke);
        std::set<uint64_t> fixedNodes;
        std::map<uint64_t, vfem::Vec3<double>> loadedNodes;
        vfem::getBoundaryConditions(modelName, fixedNodes, loadedNodes);
        if (parseOnly) {
            long long filled = 0, weighted = 0;
            for (size_t i = 0; i < model.size(); ++i) {
                filled += model[i] == 1;
                weighted += (long long)(i % 9973) * model[i];
            }
            double keSum = 0, loadSum = 0;
            for (int i = 0; i < 24; ++i)
                for (int j = 0; j < 24; ++j) keSum += Ke[i][j] * (1 + i + 24 * j);
            unsigned long long fixedSum = 0, loadIdSum = 0;
            for (uint64_t v : fixedNodes) fixedSum += v;
            for (auto& kv : loadedNodes) {
                loadIdSum += kv.first;
                loadSum += kv.second.x + 2 * kv.second.y + 3 * kv.second.z;
            }
            std::printf("dims %d %d %d\nfilled %lld\nweighted %lld\nke %.17g\nfixed %zu %llu\nloads %zu %llu %.17g\n",
                        sx, sy, sz, filled, weighted, keSum, fixedNodes.size(), fixedSum, loadedNodes.size(),
                        loadIdSum, loadSum);
            std::vector<double> sample;
            for (auto& kv : loadedNodes) sample.push_back(kv.second.z);
            vfem::saveVector(sample, modelName + "_loadz", digits);
            return 0;
        }
        auto A = vfem::assembleSystemMatrix(model.data(), sx, sy, sz, Ke, fixedNodes, numLevels, skipLevels);
        std::vector<double> f(A.rows(), 0.0), u;
        vfem::applyBoundaryConditions(f, loadedNodes, fixedNodes);
        vfem_stats st = vfem::solveWithKompute(A, f, u);
        double compliance = 0;
        for (size_t i = 0; i < f.size(); ++i) compliance += f[i] * u[i];
        std::printf("Degrees of freedom: %lld\nIterations: %lld\nCompliance: %.17g\n", (long long)A.rows(),
                    (long long)st.iterations, compliance);
        vfem::saveVector(u, modelName, digits);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
