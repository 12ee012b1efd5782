// vfem.hpp -- header-only C++ shim that re-creates the reference's solve-path
// names on top of the C ABI in vfem.h, so a reference caller (src/main.cpp of
// VulkanFEM) can switch with minimal edits.  No Eigen: vectors are
// std::vector<double>; fixed nodes are a std::set<uint64_t> and loads a
// std::map<uint64_t, Vec3> as in the reference (include/in.hpp:19-34).
//
//   reference                                   shim
//   assembleSystemMatrix<double>(...)           vfem::assembleSystemMatrix(...)   (include/FEM.hpp:33-34)
//   applyBoundaryConditions(f, loads, fixed)    vfem::applyBoundaryConditions(...) (include/FEM.hpp:63-64)
//   solveWithKompute(A, f, u)                   vfem::solveWithKompute(A, f, u)    (include/FEMGPU.hpp:11-12)
//   solveWithEigen(A, f, u)                     vfem::solveWithEigen(A, f, u)      (include/FEM.hpp:72-73)
//   MatrixFreeSparse<double> * x                vfem::MatrixFreeSparse::operator*  (MatrixFreeSparse.hpp:191-215)
//   Eigen::MultigridPreconditioner::solve(b)    vfem::MultigridPreconditioner::solve (MultigridPreconditioner.hpp:158-203)
//
// Errors: the reference returns void and relies on Eigen asserts; the shim
// throws vfem::Error carrying the vfem_status instead.
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#include "vfem.h"

namespace vfem {

struct Error : std::runtime_error {
    vfem_status status;
    Error(vfem_status s, const std::string& where)
        : std::runtime_error(where + ": " + vfem_status_string(s) + " (" + vfem_last_error_message() + ")"),
          status(s) {}
};

inline void check(vfem_status s, const char* where) {
    if (s != VFEM_OK) throw Error(s, where);
}

template <typename T>
struct Vec3 {
    T x, y, z;
};

// The assembled operator and its multigrid hierarchy, resident on the GPU.
class MatrixFreeSparse {
public:
    MatrixFreeSparse() = default;
    MatrixFreeSparse(const std::vector<uint8_t>& voxels, int nx, int ny, int nz, const double Ke[24][24],
                     const std::set<uint64_t>& fixedNodes, int numLevels, int skipLevels,
                     const float* E = nullptr) {
        std::vector<int64_t> fixed(fixedNodes.begin(), fixedNodes.end());
        vfem_problem* p = nullptr;
        check(vfem_problem_create(voxels.data(), nx, ny, nz, &Ke[0][0], E, fixed.data(), (int64_t)fixed.size(),
                                  numLevels, skipLevels, &p),
              "assembleSystemMatrix");
        handle_.reset(p, vfem_problem_destroy);
        int64_t n = 0;
        check(vfem_problem_info(p, 0, &n, nullptr, &numLevels_, nullptr), "vfem_problem_info");
        rows_ = 3 * n;
    }
    int64_t rows() const { return rows_; }
    int64_t cols() const { return rows_; }
    int numLevels() const { return numLevels_; }
    vfem_problem* handle() const { return handle_.get(); }

    // y = K x with the fixed rows zeroed (MatrixFreeSparse.hpp:197-214).
    std::vector<double> operator*(const std::vector<double>& x) const {
        std::vector<double> y(x.size());
        check(vfem_apply_operator(handle_.get(), x.data(), y.data()), "MatrixFreeSparse::operator*");
        return y;
    }

private:
    std::shared_ptr<vfem_problem> handle_;
    int64_t rows_ = 0;
    int32_t numLevels_ = 0;
};

class MultigridPreconditioner {
public:
    MultigridPreconditioner() = default;
    explicit MultigridPreconditioner(const MatrixFreeSparse& A, int mode = VFEM_MG_REFERENCE) : A_(&A), mode_(mode) {}
    MultigridPreconditioner& compute(const MatrixFreeSparse& A) {
        A_ = &A;
        return *this;
    }
    std::vector<double> solve(const std::vector<double>& b) const {
        if (!A_) throw Error(VFEM_ERR_INVALID_ARGUMENT, "MultigridPreconditioner is not initialized");
        std::vector<double> z(b.size());
        check(vfem_apply_preconditioner(A_->handle(), mode_, b.data(), z.data()), "MultigridPreconditioner::solve");
        return z;
    }

private:
    const MatrixFreeSparse* A_ = nullptr;
    int mode_ = VFEM_MG_REFERENCE;
};

inline MatrixFreeSparse assembleSystemMatrix(int* voxelModel, int nx, int ny, int nz, double Ke[24][24],
                                             const std::set<uint64_t>& fixedNodes, int numLevels, int skipLevels) {
    std::vector<uint8_t> vox((size_t)nx * ny * nz);
    for (size_t i = 0; i < vox.size(); ++i) vox[i] = voxelModel[i] == 1 ? 1 : 0;
    return MatrixFreeSparse(vox, nx, ny, nz, Ke, fixedNodes, numLevels, skipLevels);
}

// f[3*node + c] = load (src/FEM.cpp:568-584, matrix-free branch).
inline void applyBoundaryConditions(std::vector<double>& f, const std::map<uint64_t, Vec3<double>>& loadedNodes,
                                    const std::set<uint64_t>& /*fixedNodes*/) {
    for (const auto& kv : loadedNodes) {
        f[3 * kv.first] = kv.second.x;
        f[3 * kv.first + 1] = kv.second.y;
        f[3 * kv.first + 2] = kv.second.z;
    }
}

// GPU MG-PCG solve (src/FEMGPU.cpp:32-554).  Options default to the reference's
// (rtol 1e-6, additive MG, FP64); pass opt to choose another form.
inline vfem_stats solveWithKompute(const MatrixFreeSparse& A, const std::vector<double>& f, std::vector<double>& u,
                                   const vfem_options* opt = nullptr) {
    vfem_options o;
    vfem_options_default(&o);
    if (opt) o = *opt;
    check(vfem_problem_set_rhs(A.handle(), f.data()), "solveWithKompute");
    u.resize(f.size());
    vfem_stats st{};
    check(vfem_solve(A.handle(), &o, nullptr, u.data(), &st), "solveWithKompute");
    return st;
}

// The CPU Eigen path of the reference (src/FEM.cpp:589-637) maps to the same solve.
inline vfem_stats solveWithEigen(const MatrixFreeSparse& A, const std::vector<double>& f, std::vector<double>& u) {
    return solveWithKompute(A, f, u);
}

}  // namespace vfem
