// vfem_oracle.cpp -- CPU restatement of VulkanFEM's matrix-free MG-PCG path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle that the tests, the smoke
// check and the CPU-baseline leg of the benchmark compare the CUDA library
// against.  Nothing in the product library links, loads or calls it.
//
// PARITY UNPINNED: the reference ships no golden outputs and no tests, and it
// cannot be compiled here (its Eigen 3.4.0 and Kompute submodules are not
// vendored).  This restatement is pinned only by derived known-answer checks
// (element stiffness identity, fixture counts, operator symmetry, rigid modes,
// transfer-table identities) that live in tests/.
//
// Every routine follows the reference file:line given beside it (paths are
// relative to the reference project root).  Third-party arithmetic that the
// reference takes from Eigen 3.4.0 is restated from its published algorithm:
//   * Eigen::ConjugateGradient  (Eigen/src/IterativeLinearSolvers/ConjugateGradient.h,
//     3.4.0): x0 = 0, r = b, threshold = max(tol^2 |b|^2, DBL_MIN), stop on the
//     recursive residual, default max iterations 2n.
//   * Eigen::SimplicialLDLT: replaced by a banded LDL^T in natural order of the
//     free coarse DOFs (same factorisation, different fill ordering, so results
//     agree to rounding).
//
// Deliberate deviation (documented): for odd fine-level element counts the
// reference's restriction mapping linearises out-of-range stencil positions
// (FEM.cpp:350, Linearize with x == dims.x) and so can alias a node of the next
// row.  The oracle treats out-of-range stencil positions as absent (-1).  All
// benchmark configurations have even dimensions on every level, where the two
// agree exactly.

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct V3 {
    int x, y, z;
};

inline int64_t lin(int x, int y, int z, int dx, int dy) {
    return (int64_t)x + (int64_t)dx * ((int64_t)y + (int64_t)dy * z);
}

// Trilinear 1-D weight of fine local position a (0..div) to coarse local b (0/1):
// the tensor-product form of restrictionOperatorValues (RestrictionOperator.hpp:86-115,
// divider 2) and restrictionOperator4Values (RestrictionOperator.hpp:117-244, divider 4).
inline double tri1(int a, int b, int div) {
    return b == 0 ? double(div - a) / div : double(a) / div;
}

struct Level {
    int ex = 0, ey = 0, ez = 0;          // levelDims (FEM.cpp:246,256-260)
    std::vector<V3> elements;            // levelElements, sorted by linear index
    std::vector<double> elemE;           // modulus multiplier per element (extension; 1 in the reference)
    std::vector<int64_t> nodes;          // used node linear ids in the node grid, sorted
    std::vector<int32_t> lookup;         // node grid linear id -> compressed id (or -1)
    std::vector<std::array<int, 4>> e2n; // elementToNode, 4 columns (FEM.cpp:188-198,332,345)
    std::vector<double> invDiag;         // invDiagKOnLevels (FEM.cpp:250,463)
    std::vector<int64_t> fixed;          // fixedNodesInLevels, sorted compressed ids
    // Transfer data attached to a coarse level i (reference index i-1):
    int divider = 2;                     // FEM.cpp:266-272
    int nb = 27;                         // bounding nodes per coarse element (27 or 125)
    std::vector<int32_t> mapping;        // restrictionMappings[i-1] (FEM.cpp:348-362)
    // Attached to the fine level i-1 of a transfer:
    std::vector<double> W;               // restrictionCoefficients[i-1] (FEM.cpp:400)
    int64_t ndof() const { return 3 * (int64_t)nodes.size(); }
    int nx() const { return ex + 1; }
    int ny() const { return ey + 1; }
    int nz() const { return ez + 1; }
};

struct Problem {
    int numLevels = 1, skipLevels = 0;
    double Ke[24][24];                   // symmetrised element stiffness (FEM.cpp:200-210)
    std::vector<Level> L;
    // coarsest solve
    std::vector<int64_t> coarseFreeDoFs; // FEM.cpp:473-496
    int64_t nc = 0;                      // free coarse DOFs
    int64_t bw = 0;                      // half bandwidth of Kc in natural order
    std::vector<double> band;            // LDL^T factor, band storage [i][bw+1]: L(i, i-k) at k
    bool floatCoeffs = false;            // FEMGPU.cpp:226-242 (float W and invDiag)
    int threads = 1;
};

// ---------------------------------------------------------------- tables
// restrictionOnElementValues / restrictionOnElement4Values
// (RestrictionOperator.hpp:6-16,18-84): local node a (x fastest) of child
// element ch inside the (div+1)^3 bounding-node stencil.
int childNode(int ch, int a, int div) {
    int cx = ch % div, cy = (ch / div) % div, cz = ch / (div * div);
    int ax = a & 1, ay = (a >> 1) & 1, az = (a >> 2) & 1;
    int n = div + 1;
    return (cx + ax) + n * ((cy + ay) + n * (cz + az));
}

// Diagonal of the Galerkin element matrix R_DOF^T (Ke placed at child ch) R_DOF
// (FEM.cpp:365-395 with restrictionOperatorDoFValues / restrictionOperatorDoF4Values,
// RestrictionOperator.hpp:246-708).  Only the diagonal is ever used
// (GetInverseDiagonal, FEM.cpp:124-151), so only the diagonal is formed; the
// Galerkin sum is linear in the children, so it is accumulated child by child.
void childDiag(const double Ke[24][24], int div, std::vector<double>& tab) {
    int nch = div * div * div;
    int n = div + 1;
    tab.assign((size_t)nch * 24, 0.0);
    for (int ch = 0; ch < nch; ++ch) {
        for (int k = 0; k < 24; ++k) {
            int C = k / 3, c = k % 3;
            int bx = C & 1, by = (C >> 1) & 1, bz = (C >> 2) & 1;
            double s = 0.0;
            for (int k1 = 0; k1 < 24; ++k1) {
                if (k1 % 3 != c) continue;
                int f1 = childNode(ch, k1 / 3, div);
                int f1x = f1 % n, f1y = (f1 / n) % n, f1z = f1 / (n * n);
                double r1 = tri1(f1x, bx, div) * tri1(f1y, by, div) * tri1(f1z, bz, div);
                if (r1 == 0.0) continue;
                for (int k2 = 0; k2 < 24; ++k2) {
                    if (k2 % 3 != c) continue;
                    int f2 = childNode(ch, k2 / 3, div);
                    int f2x = f2 % n, f2y = (f2 / n) % n, f2z = f2 / (n * n);
                    double r2 = tri1(f2x, bx, div) * tri1(f2y, by, div) * tri1(f2z, bz, div);
                    s += r1 * Ke[k1][k2] * r2;
                }
            }
            tab[(size_t)ch * 24 + k] = s;
        }
    }
}

// ---------------------------------------------------------------- assembly
// EnlistUsedElements (FEM.cpp:66-100) + compressed numbering (FEM.cpp:179-186).
void buildFinest(Problem& P, const int32_t* vox, int sx, int sy, int sz, const float* E) {
    Level& l = P.L[0];
    l.ex = sx; l.ey = sy; l.ez = sz;
    int nx = sx + 1, ny = sy + 1, nz = sz + 1;
    for (int z = 0; z < sz; ++z)
        for (int y = 0; y < sy; ++y)
            for (int x = 0; x < sx; ++x)
                if (vox[lin(x, y, z, sx, sy)] == 1) {
                    l.elements.push_back({x, y, z});
                    l.elemE.push_back(E ? (double)E[lin(x, y, z, sx, sy)] : 1.0);
                }
    l.lookup.assign((size_t)nx * ny * nz, -1);
    std::vector<uint8_t> used((size_t)nx * ny * nz, 0);
    for (auto& e : l.elements)
        for (int dz = 0; dz < 2; ++dz)
            for (int dy = 0; dy < 2; ++dy)
                for (int dx = 0; dx < 2; ++dx) used[lin(e.x + dx, e.y + dy, e.z + dz, nx, ny)] = 1;
    for (int64_t i = 0; i < (int64_t)used.size(); ++i)
        if (used[i]) { l.lookup[i] = (int32_t)l.nodes.size(); l.nodes.push_back(i); }
    // elementToGlobal: column j = y + 2z holds node (ex, ey+y, ez+z); the +x
    // neighbour is implicitly index+1 (FEM.cpp:188-198).
    l.e2n.resize(l.elements.size());
    for (size_t i = 0; i < l.elements.size(); ++i) {
        auto& e = l.elements[i];
        for (int z = 0; z < 2; ++z)
            for (int y = 0; y < 2; ++y)
                l.e2n[i][y + 2 * z] = l.lookup[lin(e.x, e.y + y, e.z + z, nx, ny)];
    }
}

// GetInverseDiagonal (FEM.cpp:105-151).
void inverseDiagonal(Level& l, double scale, const double Ke[24][24],
                     const std::vector<std::vector<double>>* unique) {
    std::vector<double> diag(l.ndof(), 0.0);
    for (size_t i = 0; i < l.e2n.size(); ++i) {
        for (int k = 0; k < 24; ++k) {
            int64_t dof = 3 * (int64_t)l.e2n[i][k / 6] + (k % 6);
            double d = (unique && !(*unique)[i].empty()) ? (*unique)[i][k] : scale * l.elemE[i] * Ke[k][k];
            diag[dof] += d;
        }
    }
    l.invDiag.resize(diag.size());
    for (size_t i = 0; i < diag.size(); ++i) l.invDiag[i] = 1.0 / diag[i];
}

// Restrict (fine level `lv`) -> coarse level lv+1 (MultigridPreconditioner.hpp:67-108).
void restrictVec(const Problem& P, int lv, const double* r, double* out, bool useW = true);

// MG levels loop (FEM.cpp:223-471).
void buildLevels(Problem& P, int numLevels) {
    std::vector<double> tab2, tab4;
    childDiag(P.Ke, 2, tab2);
    childDiag(P.Ke, 4, tab4);
    for (int i = 1; i < numLevels; ++i) {
        Level& f = P.L[i - 1];
        Level c;
        c.ex = f.ex / 2 + f.ex % 2;
        c.ey = f.ey / 2 + f.ey % 2;
        c.ez = f.ez / 2 + f.ez % 2;
        int div = 2;
        if (i == 1 && P.skipLevels > 0) div = 1 << (P.skipLevels + 1);
        int nch = div * div * div;
        c.divider = div;
        c.nb = (div + 1) * (div + 1) * (div + 1);
        // Coarse elements and children counts (FEM.cpp:274-283).  The coarse
        // element grid used for linearisation has dims c.ex.. (levelDims[i]).
        int64_t ncell = (int64_t)c.ex * c.ey * c.ez;
        std::vector<int32_t> childCount(ncell, 0);
        std::vector<std::vector<std::pair<int, double>>> childList(ncell);  // (child slot, modulus)
        for (size_t fi = 0; fi < f.elements.size(); ++fi) {
            const V3& fe = f.elements[fi];
            int x = fe.x / div, y = fe.y / div, z = fe.z / div;
            int64_t id = lin(x, y, z, c.ex, c.ey);
            int chx = fe.x - x * div, chy = fe.y - y * div, chz = fe.z - z * div;
            childList[id].push_back({chx + div * (chy + div * chz), f.elemE[fi]});
            childCount[id]++;
        }
        for (int z = 0; z < c.ez; ++z)
            for (int y = 0; y < c.ey; ++y)
                for (int x = 0; x < c.ex; ++x) {
                    int64_t id = lin(x, y, z, c.ex, c.ey);
                    if (childCount[id] == 0) continue;
                    c.elements.push_back({x, y, z});
                    // Extension: a coarse element carries the mean modulus of its used children.
                    double s = 0.0;
                    for (auto& ch : childList[id]) s += ch.second;
                    c.elemE.push_back((double)(float)(s / childCount[id]));
                }
        // Coarse nodes and numbering (FEM.cpp:291-319).
        int cnx = c.nx(), cny = c.ny(), cnz = c.nz();
        std::vector<uint8_t> used((size_t)cnx * cny * cnz, 0);
        for (auto& e : c.elements)
            for (int dz = 0; dz < 2; ++dz)
                for (int dy = 0; dy < 2; ++dy)
                    for (int dx = 0; dx < 2; ++dx) used[lin(e.x + dx, e.y + dy, e.z + dz, cnx, cny)] = 1;
        c.lookup.assign(used.size(), -1);
        for (int64_t k = 0; k < (int64_t)used.size(); ++k)
            if (used[k]) { c.lookup[k] = (int32_t)c.nodes.size(); c.nodes.push_back(k); }
        // elementToGlobalOnLevel, restrictionMapping, restriction counts,
        // Galerkin diagonals of partially filled coarse elements (FEM.cpp:340-396).
        int fnx = f.nx(), fny = f.ny(), fnz = f.nz();
        int nbAxis = div + 1;
        size_t ne = c.elements.size();
        c.e2n.resize(ne);
        c.mapping.assign(ne * c.nb, -1);
        std::vector<double> count(f.ndof(), 0.0);
        std::vector<std::vector<double>> unique(ne);
        const std::vector<double>& tab = (div == 4) ? tab4 : tab2;
        double childScale = std::pow(2.0, i - 1);
        for (size_t ie = 0; ie < ne; ++ie) {
            auto& e = c.elements[ie];
            for (int z = 0; z < 2; ++z)
                for (int y = 0; y < 2; ++y) c.e2n[ie][y + 2 * z] = c.lookup[lin(e.x, e.y + y, e.z + z, cnx, cny)];
            for (int nz_ = 0; nz_ < nbAxis; ++nz_)
                for (int ny_ = 0; ny_ < nbAxis; ++ny_)
                    for (int nx_ = 0; nx_ < nbAxis; ++nx_) {
                        int gx = e.x * div + nx_, gy = e.y * div + ny_, gz = e.z * div + nz_;
                        int slot = nx_ + nbAxis * (ny_ + nbAxis * nz_);
                        if (gx >= fnx || gy >= fny || gz >= fnz) continue;  // see header note
                        int32_t id = f.lookup[lin(gx, gy, gz, fnx, fny)];
                        if (id < 0) continue;
                        c.mapping[ie * c.nb + slot] = id;
                        count[3 * (int64_t)id] += 1.0;
                        count[3 * (int64_t)id + 1] += 1.0;
                        count[3 * (int64_t)id + 2] += 1.0;
                    }
            int64_t cell = lin(e.x, e.y, e.z, c.ex, c.ey);
            if (childCount[cell] < nch) {
                std::vector<double> d(24, 0.0);
                for (auto& ch : childList[cell])
                    for (int k = 0; k < 24; ++k) d[k] += childScale * ch.second * tab[(size_t)ch.first * 24 + k];
                unique[ie] = d;
            }
        }
        f.W.resize(count.size());
        for (size_t k = 0; k < count.size(); ++k) f.W[k] = 1.0 / count[k];  // cwiseInverse (FEM.cpp:400)
        P.L.push_back(std::move(c));
        Level& cl = P.L.back();
        Level& fl = P.L[i - 1];
        // Fixed nodes of this level: restrict an indicator of the fine fixed
        // nodes and keep every node with a non-zero entry (FEM.cpp:402-460).
        {
            std::vector<double> ind(fl.ndof(), 0.0);
            for (int64_t n : fl.fixed) ind[3 * n] = ind[3 * n + 1] = ind[3 * n + 2] = 1.0;
            std::vector<double> res(cl.ndof(), 0.0);
            restrictVec(P, i - 1, ind.data(), res.data());
            for (int64_t k = 0; k < (int64_t)res.size(); ++k) {
                int64_t n = k / 3;
                if (res[k] != 0.0 && (cl.fixed.empty() || cl.fixed.back() != n)) cl.fixed.push_back(n);
            }
        }
        inverseDiagonal(cl, std::pow(2.0, i + P.skipLevels), P.Ke, &unique);
        if (cl.ex <= 2 || cl.ey <= 2 || cl.ez <= 2) {  // FEM.cpp:465-470
            numLevels = i + 1;
            break;
        }
    }
    P.numLevels = (int)P.L.size();
}

void restrictVec(const Problem& P, int lv, const double* r, double* out, bool useW) {
    const Level& f = P.L[lv];
    const Level& c = P.L[lv + 1];
    int div = c.divider, n = div + 1;
    std::fill(out, out + c.ndof(), 0.0);
    std::vector<double> tempR(f.ndof());
#pragma omp parallel for num_threads(P.threads) schedule(static) if (P.threads > 1)
    for (int64_t k = 0; k < f.ndof(); ++k) {
        double w = useW ? f.W[k] : 1.0;
        if (P.floatCoeffs) w = (double)(float)w;
        tempR[k] = r[k] * w;
    }
    auto body = [&](size_t ie) {
        for (int a = 0; a < 8; ++a) {
            int64_t cn = (int64_t)c.e2n[ie][a >> 1] + (a & 1);  // xInd/offset (MultigridPreconditioner.hpp:86-87)
            int bx = a & 1, by = (a >> 1) & 1, bz = (a >> 2) & 1;
            double acc[3] = {0, 0, 0};
            for (int s = 0; s < c.nb; ++s) {
                int32_t m = c.mapping[ie * c.nb + s];
                if (m < 0) continue;  // mask
                int sx = s % n, sy = (s / n) % n, sz = s / (n * n);
                double w = tri1(sx, bx, div) * tri1(sy, by, div) * tri1(sz, bz, div);
                for (int cc = 0; cc < 3; ++cc) acc[cc] += tempR[3 * (int64_t)m + cc] * w;
            }
            for (int cc = 0; cc < 3; ++cc) out[3 * cn + cc] += acc[cc];
        }
    };
    if (P.threads > 1) {
        // 8-colouring by coarse element parity: same-colour elements share no node.
        for (int col = 0; col < 8; ++col) {
#pragma omp parallel for num_threads(P.threads) schedule(static)
            for (int64_t ie = 0; ie < (int64_t)c.elements.size(); ++ie) {
                const V3& e = c.elements[ie];
                if (((e.x & 1) | ((e.y & 1) << 1) | ((e.z & 1) << 2)) == col) body(ie);
            }
        }
    } else {
        for (size_t ie = 0; ie < c.elements.size(); ++ie) body(ie);
    }
}

// interpolate (MultigridPreconditioner.hpp:110-155): W o sum_e R x_c[e], with the
// "overRow" sink for unused stencil positions.
void interpolateVec(const Problem& P, int lv, const double* xc, double* out) {
    const Level& f = P.L[lv];
    const Level& c = P.L[lv + 1];
    int div = c.divider, n = div + 1;
    std::fill(out, out + f.ndof(), 0.0);
    auto body = [&](size_t ie) {
        for (int s = 0; s < c.nb; ++s) {
            int32_t m = c.mapping[ie * c.nb + s];
            if (m < 0) continue;  // overRow sink
            int sx = s % n, sy = (s / n) % n, sz = s / (n * n);
            double acc[3] = {0, 0, 0};
            for (int a = 0; a < 8; ++a) {
                int64_t cn = (int64_t)c.e2n[ie][a >> 1] + (a & 1);
                int bx = a & 1, by = (a >> 1) & 1, bz = (a >> 2) & 1;
                double w = tri1(sx, bx, div) * tri1(sy, by, div) * tri1(sz, bz, div);
                for (int cc = 0; cc < 3; ++cc) acc[cc] += w * xc[3 * cn + cc];
            }
            for (int cc = 0; cc < 3; ++cc) out[3 * (int64_t)m + cc] += acc[cc];
        }
    };
    if (P.threads > 1) {
        for (int col = 0; col < 8; ++col) {
#pragma omp parallel for num_threads(P.threads) schedule(static)
            for (int64_t ie = 0; ie < (int64_t)c.elements.size(); ++ie) {
                const V3& e = c.elements[ie];
                if (((e.x & 1) | ((e.y & 1) << 1) | ((e.z & 1) << 2)) == col) body(ie);
            }
        }
    } else {
        for (size_t ie = 0; ie < c.elements.size(); ++ie) body(ie);
    }
#pragma omp parallel for num_threads(P.threads) schedule(static) if (P.threads > 1)
    for (int64_t k = 0; k < f.ndof(); ++k) {
        double w = f.W[k];
        if (P.floatCoeffs) w = (double)(float)w;
        out[k] *= w;
    }
}

// Coarsest level: free DoFs (FEM.cpp:473-496), explicit Kc with
// 2^(L-1+skip) Ke (assembleK, FEM.cpp:19-63,498-513), factorised once
// (SimplicialLDLT, MultigridPreconditioner.hpp:39-53) -- here a banded LDL^T.
void buildCoarse(Problem& P) {
    Level& l = P.L.back();
    std::vector<int64_t> freeIdx(l.nodes.size(), -1);
    size_t fi = 0;
    int64_t nfree = 0;
    for (int64_t n = 0; n < (int64_t)l.nodes.size(); ++n) {
        while (fi < l.fixed.size() && l.fixed[fi] < n) ++fi;
        bool isFixed = fi < l.fixed.size() && l.fixed[fi] == n;
        if (!isFixed) freeIdx[n] = nfree++;
    }
    P.coarseFreeDoFs.clear();
    for (int64_t n = 0; n < (int64_t)l.nodes.size(); ++n)
        if (freeIdx[n] >= 0)
            for (int c = 0; c < 3; ++c) P.coarseFreeDoFs.push_back(3 * n + c);
    int64_t N = 3 * nfree;
    P.nc = N;
    double mult = std::pow(2.0, P.numLevels + P.skipLevels - 1);
    // bandwidth
    int64_t bw = 0;
    auto nodeOf = [&](const V3& e, int a) -> int64_t {
        int dx = a & 1, dy = (a >> 1) & 1, dz = (a >> 2) & 1;
        return freeIdx[l.lookup[lin(e.x + dx, e.y + dy, e.z + dz, l.nx(), l.ny())]];
    };
    for (auto& e : l.elements) {
        int64_t lo = INT64_MAX, hi = -1;
        for (int a = 0; a < 8; ++a) {
            int64_t g = nodeOf(e, a);
            if (g < 0) continue;
            lo = std::min(lo, g);
            hi = std::max(hi, g);
        }
        if (hi >= 0) bw = std::max(bw, 3 * (hi - lo) + 2);
    }
    P.bw = bw;
    int64_t W = bw + 1;
    P.band.assign((size_t)N * W, 0.0);  // band[i*W + k] = A(i, i-k), k <= bw
    for (size_t ie = 0; ie < l.elements.size(); ++ie) {
        const V3& e = l.elements[ie];
        const double me = mult * l.elemE[ie];
        for (int a = 0; a < 8; ++a) {
            int64_t ga = nodeOf(e, a);
            if (ga < 0) continue;
            for (int b = 0; b < 8; ++b) {
                int64_t gb = nodeOf(e, b);
                if (gb < 0) continue;
                for (int c1 = 0; c1 < 3; ++c1)
                    for (int c2 = 0; c2 < 3; ++c2) {
                        int64_t i = 3 * ga + c1, j = 3 * gb + c2;
                        if (j > i) continue;
                        P.band[(size_t)i * W + (i - j)] += me * P.Ke[3 * a + c1][3 * b + c2];
                    }
            }
        }
    }
    // In-place banded LDL^T: A = L D L^T, L unit lower; store D on k = 0.
    std::vector<double> tmp(W);
    for (int64_t j = 0; j < N; ++j) {
        int64_t k0 = std::max<int64_t>(0, j - bw);
        // tmp[p] = L(j,p) * D(p) for p in [k0, j)
        double d = P.band[(size_t)j * W];
        for (int64_t p = k0; p < j; ++p) {
            double ljp = P.band[(size_t)j * W + (j - p)];
            double v = ljp * P.band[(size_t)p * W];
            tmp[j - p] = v;
            d -= ljp * v;
        }
        P.band[(size_t)j * W] = d;
        int64_t iend = std::min<int64_t>(N, j + bw + 1);
        for (int64_t i = j + 1; i < iend; ++i) {
            double s = P.band[(size_t)i * W + (i - j)];
            int64_t p0 = std::max<int64_t>(k0, i - bw);
            for (int64_t p = p0; p < j; ++p) s -= P.band[(size_t)i * W + (i - p)] * tmp[j - p];
            P.band[(size_t)i * W + (i - j)] = s / d;
        }
    }
}

void coarseSolve(const Problem& P, const double* rhs, double* x) {
    int64_t N = P.nc, bw = P.bw, W = bw + 1;
    std::vector<double> y(rhs, rhs + N);
    for (int64_t i = 0; i < N; ++i) {
        double s = y[i];
        for (int64_t p = std::max<int64_t>(0, i - bw); p < i; ++p) s -= P.band[(size_t)i * W + (i - p)] * y[p];
        y[i] = s;
    }
    for (int64_t i = 0; i < N; ++i) y[i] /= P.band[(size_t)i * W];
    for (int64_t i = N - 1; i >= 0; --i) {
        double s = y[i];
        int64_t pend = std::min<int64_t>(N, i + bw + 1);
        for (int64_t p = i + 1; p < pend; ++p) s -= P.band[(size_t)p * W + (p - i)] * y[p];
        y[i] = s;
    }
    std::copy(y.begin(), y.end(), x);
}

// MatrixFreeSparse product scaleAndAddTo (MatrixFreeSparse.hpp:197-214), alpha = 1
// into a zeroed destination (Eigen evalTo), then the fixed rows are zeroed.
void matvec(const Problem& P, const double* x, double* y) {
    const Level& l = P.L[0];
    std::fill(y, y + l.ndof(), 0.0);
    auto body = [&](size_t i) {
        int64_t xs[24];
        for (int k = 0; k < 24; ++k) xs[k] = 3 * (int64_t)l.e2n[i][k / 6] + (k % 6);
        double xe[24];
        for (int k = 0; k < 24; ++k) xe[k] = x[xs[k]];
        for (int r = 0; r < 24; ++r) {
            double s = 0.0;
            for (int k = 0; k < 24; ++k) s += P.Ke[r][k] * xe[k];
            y[xs[r]] += l.elemE[i] * s;
        }
    };
    if (P.threads > 1) {
        for (int col = 0; col < 8; ++col) {
#pragma omp parallel for num_threads(P.threads) schedule(static)
            for (int64_t i = 0; i < (int64_t)l.elements.size(); ++i) {
                const V3& e = l.elements[i];
                if (((e.x & 1) | ((e.y & 1) << 1) | ((e.z & 1) << 2)) == col) body(i);
            }
        }
    } else {
        for (size_t i = 0; i < l.elements.size(); ++i) body(i);
    }
    for (int64_t n : l.fixed) y[3 * n] = y[3 * n + 1] = y[3 * n + 2] = 0.0;
}

// MultigridPreconditioner::_solve_impl (MultigridPreconditioner.hpp:158-193).
void precond(const Problem& P, const double* b, double* out) {
    int nl = P.numLevels;
    std::vector<std::vector<double>> xs(nl), rs(nl);
    rs[0].assign(b, b + P.L[0].ndof());
    xs[0].assign(P.L[0].ndof(), 0.0);
    auto dinv = [&](int lv, int64_t k) {
        double v = P.L[lv].invDiag[k];
        return P.floatCoeffs ? (double)(float)v : v;
    };
    for (int i = 0; i < nl - 1; ++i) {
#pragma omp parallel for num_threads(P.threads) schedule(static) if (P.threads > 1)
        for (int64_t k = 0; k < P.L[i].ndof(); ++k) xs[i][k] += rs[i][k] * dinv(i, k);  // smooth
        rs[i + 1].assign(P.L[i + 1].ndof(), 0.0);
        restrictVec(P, i, rs[i].data(), rs[i + 1].data());
        xs[i + 1].assign(P.L[i + 1].ndof(), 0.0);
    }
    {
        std::vector<double> rhs(P.nc), sol(P.nc);
        for (int64_t k = 0; k < P.nc; ++k) rhs[k] = rs[nl - 1][P.coarseFreeDoFs[k]];
        coarseSolve(P, rhs.data(), sol.data());
        for (int64_t k = 0; k < P.nc; ++k) xs[nl - 1][P.coarseFreeDoFs[k]] = sol[k];
    }
    for (int i = nl - 1; i > 0; --i) {
        std::vector<double> t(P.L[i - 1].ndof());
        interpolateVec(P, i - 1, xs[i].data(), t.data());
#pragma omp parallel for num_threads(P.threads) schedule(static) if (P.threads > 1)
        for (int64_t k = 0; k < P.L[i - 1].ndof(); ++k) xs[i - 1][k] += t[k];
#pragma omp parallel for num_threads(P.threads) schedule(static) if (P.threads > 1)
        for (int64_t k = 0; k < P.L[i - 1].ndof(); ++k) xs[i - 1][k] += rs[i - 1][k] * dinv(i - 1, k);
    }
    std::copy(xs[0].begin(), xs[0].end(), out);
    for (int64_t n : P.L[0].fixed) out[3 * n] = out[3 * n + 1] = out[3 * n + 2] = 0.0;
}

double dot(const Problem& P, const double* a, const double* b, int64_t n) {
    double s = 0.0;
    if (P.threads > 1) {
#pragma omp parallel for num_threads(P.threads) reduction(+ : s) schedule(static)
        for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
    } else {
        for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
    }
    return s;
}

}  // namespace

extern "C" {

struct OracleProblem;

// assembleSystemMatrix<double> (FEM.cpp:157-554) with the MATRIX_FREE and
// MULTIGRID definitions.  voxels: int32 occupancy (1 = filled), x fastest,
// dims (sx, sy, sz).  Ke: 24x24 row-major; only its upper triangle is read
// (FEM.cpp:200-210).  fixed: compressed node ids (0-based).
// Extension with no reference counterpart: E (per voxel, same layout as the
// voxels, or null) multiplies the element stiffness; coarse elements carry the
// mean modulus of their used children.  With E null the reference is unchanged.
OracleProblem* oracle_create_e(const int32_t* voxels, int sx, int sy, int sz, const double* Ke, const float* E,
                               const int64_t* fixed, int64_t nfixed, int numLevels, int skipLevels) {
    if (skipLevels < 0 || skipLevels > 1 || numLevels < 1) return nullptr;
    Problem* P = new Problem();
    P->skipLevels = skipLevels;
    for (int i = 0; i < 24; ++i) {
        P->Ke[i][i] = Ke[i * 24 + i];
        for (int j = 0; j < i; ++j) P->Ke[i][j] = P->Ke[j][i] = Ke[j * 24 + i];
    }
    P->L.resize(1);
    buildFinest(*P, voxels, sx, sy, sz, E);
    std::vector<int64_t> fx(fixed, fixed + nfixed);
    std::sort(fx.begin(), fx.end());
    fx.erase(std::unique(fx.begin(), fx.end()), fx.end());
    P->L[0].fixed = fx;
    inverseDiagonal(P->L[0], 1.0, P->Ke, nullptr);
    buildLevels(*P, numLevels);
    buildCoarse(*P);
    return (OracleProblem*)P;
}

OracleProblem* oracle_create(const int32_t* voxels, int sx, int sy, int sz, const double* Ke,
                             const int64_t* fixed, int64_t nfixed, int numLevels, int skipLevels) {
    return oracle_create_e(voxels, sx, sy, sz, Ke, nullptr, fixed, nfixed, numLevels, skipLevels);
}

void oracle_destroy(OracleProblem* p) { delete (Problem*)p; }
void oracle_set_threads(OracleProblem* p, int t) { ((Problem*)p)->threads = t < 1 ? 1 : t; }
void oracle_set_float_coeffs(OracleProblem* p, int on) { ((Problem*)p)->floatCoeffs = on != 0; }
int oracle_num_levels(OracleProblem* p) { return ((Problem*)p)->numLevels; }
int64_t oracle_num_dofs(OracleProblem* p, int lv) { return ((Problem*)p)->L[lv].ndof(); }
int64_t oracle_num_elements(OracleProblem* p, int lv) { return (int64_t)((Problem*)p)->L[lv].elements.size(); }
int64_t oracle_num_fixed(OracleProblem* p, int lv) { return (int64_t)((Problem*)p)->L[lv].fixed.size(); }
int64_t oracle_num_coarse_free(OracleProblem* p) { return ((Problem*)p)->nc; }
void oracle_level_dims(OracleProblem* p, int lv, int32_t* out3) {
    auto& l = ((Problem*)p)->L[lv];
    out3[0] = l.ex; out3[1] = l.ey; out3[2] = l.ez;
}
// Node-grid linear ids (x fastest over (ex+1, ey+1, ez+1)) of the used nodes, in
// compressed order.
void oracle_nodes(OracleProblem* p, int lv, int64_t* out) {
    auto& l = ((Problem*)p)->L[lv];
    std::copy(l.nodes.begin(), l.nodes.end(), out);
}
void oracle_fixed(OracleProblem* p, int lv, int64_t* out) {
    auto& l = ((Problem*)p)->L[lv];
    std::copy(l.fixed.begin(), l.fixed.end(), out);
}
void oracle_inv_diag(OracleProblem* p, int lv, double* out) {
    auto& l = ((Problem*)p)->L[lv];
    std::copy(l.invDiag.begin(), l.invDiag.end(), out);
}
void oracle_restriction_coeffs(OracleProblem* p, int lv, double* out) {
    auto& l = ((Problem*)p)->L[lv];
    std::copy(l.W.begin(), l.W.end(), out);
}
void oracle_element_to_node(OracleProblem* p, int lv, int32_t* out) {
    auto& l = ((Problem*)p)->L[lv];
    for (size_t i = 0; i < l.e2n.size(); ++i)
        for (int k = 0; k < 4; ++k) out[4 * i + k] = l.e2n[i][k];
}
void oracle_matvec(OracleProblem* p, const double* x, double* y) { matvec(*(Problem*)p, x, y); }
void oracle_precond(OracleProblem* p, const double* r, double* z) { precond(*(Problem*)p, r, z); }
void oracle_restrict(OracleProblem* p, int lv, const double* in, double* out) {
    restrictVec(*(Problem*)p, lv, in, out);
}
void oracle_interpolate(OracleProblem* p, int lv, const double* in, double* out) {
    interpolateVec(*(Problem*)p, lv, in, out);
}
void oracle_coarse_solve(OracleProblem* p, const double* rhs, double* x) { coarseSolve(*(Problem*)p, rhs, x); }

// applyBoundaryConditions (FEM.cpp:568-584), MATRIX_FREE branch: f[3i+c] = load.
void oracle_apply_loads(OracleProblem* p, const int64_t* nodes, const double* loads, int64_t n, double* f) {
    (void)p;
    for (int64_t k = 0; k < n; ++k)
        for (int c = 0; c < 3; ++c) f[3 * nodes[k] + c] = loads[3 * k + c];
}

// Eigen 3.4 ConjugateGradient with MultigridPreconditioner (FEM.cpp:589-637).
// max_iter <= 0 means Eigen's default 2n.  Returns the iteration count as Eigen
// reports it; *err = sqrt(|r|^2 / |b|^2) of the recursive residual.
// iter_cap > 0 stops after that many loop passes (benchmark sampling only).
int64_t oracle_pcg(OracleProblem* p, const double* b, double* x, double tol, int64_t max_iter,
                   int use_mg, double* err, int64_t iter_cap) {
    Problem& P = *(Problem*)p;
    int64_t n = P.L[0].ndof();
    if (max_iter <= 0) max_iter = 2 * n;
    std::vector<double> r(b, b + n), pv(n), z(n), tmp(n);
    std::fill(x, x + n, 0.0);
    double rhsNorm2 = dot(P, b, b, n);
    if (rhsNorm2 == 0.0) { *err = 0.0; return 0; }
    double threshold = std::max(tol * tol * rhsNorm2, std::numeric_limits<double>::min());
    double resNorm2 = dot(P, r.data(), r.data(), n);
    if (resNorm2 < threshold) { *err = std::sqrt(resNorm2 / rhsNorm2); return 0; }
    auto M = [&](const double* in, double* out) {
        if (use_mg) precond(P, in, out);
        else std::copy(in, in + n, out);
    };
    M(r.data(), pv.data());
    double absNew = dot(P, r.data(), pv.data(), n);
    int64_t i = 0;
    while (i < max_iter) {
        matvec(P, pv.data(), tmp.data());
        double alpha = absNew / dot(P, pv.data(), tmp.data(), n);
#pragma omp parallel for num_threads(P.threads) schedule(static) if (P.threads > 1)
        for (int64_t k = 0; k < n; ++k) x[k] += alpha * pv[k];
#pragma omp parallel for num_threads(P.threads) schedule(static) if (P.threads > 1)
        for (int64_t k = 0; k < n; ++k) r[k] -= alpha * tmp[k];
        resNorm2 = dot(P, r.data(), r.data(), n);
        if (resNorm2 < threshold) break;
        if (iter_cap > 0 && i + 1 >= iter_cap) { ++i; break; }
        M(r.data(), z.data());
        double absOld = absNew;
        absNew = dot(P, r.data(), z.data(), n);
        double beta = absNew / absOld;
#pragma omp parallel for num_threads(P.threads) schedule(static) if (P.threads > 1)
        for (int64_t k = 0; k < n; ++k) pv[k] = z[k] + beta * pv[k];
        ++i;
    }
    *err = std::sqrt(resNorm2 / rhsNorm2);
    return i;
}

}  // extern "C"
