// setup.cpp -- host-side pieces of the set-up: the element stiffness and its
// Walsh-basis factorisation, the per-child Galerkin diagonal tables, and the
// plan of the level grids.  The per-node hierarchy itself is built on the
// device (setup_gpu.cu).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "vfem_internal.h"

namespace vfem {

const int kPatRow[45] = {
    3, 3, 3, 7, 7, 7, 14, 14, 14,          // class 0: normal strains
    6, 6, 4, 4, 23,                        // class (1,1,0)
    12, 12, 5, 5, 22,                      // class (1,0,1)
    13, 13, 8, 8, 21,                      // class (0,1,1)
    10, 10, 17, 17,                        // class (1,0,0)
    9, 9, 20, 20,                          // class (0,1,0)
    15, 15, 19, 19,                        // class (0,0,1)
    18, 18, 18, 16, 16, 16, 11, 11, 11};   // class (1,1,1)
const int kPatCol[45] = {
    3, 7, 14, 3, 7, 14, 3, 7, 14,
    6, 4, 6, 4, 23,
    12, 5, 12, 5, 22,
    13, 8, 13, 8, 21,
    10, 17, 10, 17,
    9, 20, 9, 20,
    15, 19, 15, 19,
    18, 16, 11, 18, 16, 11, 18, 16, 11};

void hex8Stiffness(double E, double nu, double* Ke) {
    double lam = E * nu / ((1 + nu) * (1 - 2 * nu));
    double mu = E / (2 * (1 + nu));
    double D[6][6] = {};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) D[i][j] = lam + (i == j ? 2 * mu : 0.0);
    D[3][3] = D[4][4] = D[5][5] = mu;
    std::memset(Ke, 0, 576 * sizeof(double));
    const double g[2] = {-1.0 / std::sqrt(3.0), 1.0 / std::sqrt(3.0)};
    for (int gz = 0; gz < 2; ++gz)
        for (int gy = 0; gy < 2; ++gy)
            for (int gx = 0; gx < 2; ++gx) {
                double xi[3] = {(g[gx] + 1) / 2, (g[gy] + 1) / 2, (g[gz] + 1) / 2};
                double B[6][24] = {};
                for (int a = 0; a < 8; ++a) {
                    int dx = a & 1, dy = (a >> 1) & 1, dz = (a >> 2) & 1;
                    double fx = dx ? xi[0] : 1 - xi[0], fy = dy ? xi[1] : 1 - xi[1], fz = dz ? xi[2] : 1 - xi[2];
                    double d0 = (dx ? 1 : -1) * fy * fz, d1 = fx * (dy ? 1 : -1) * fz, d2 = fx * fy * (dz ? 1 : -1);
                    B[0][3 * a] = d0;
                    B[1][3 * a + 1] = d1;
                    B[2][3 * a + 2] = d2;
                    B[3][3 * a] = d1; B[3][3 * a + 1] = d0;
                    B[4][3 * a + 1] = d2; B[4][3 * a + 2] = d1;
                    B[5][3 * a] = d2; B[5][3 * a + 2] = d0;
                }
                for (int i = 0; i < 24; ++i)
                    for (int j = 0; j < 24; ++j) {
                        double s = 0;
                        for (int p = 0; p < 6; ++p)
                            for (int q = 0; q < 6; ++q) s += B[p][i] * D[p][q] * B[q][j];
                        Ke[i * 24 + j] += s / 8.0;
                    }
            }
    for (int i = 0; i < 24; ++i)
        for (int j = 0; j < i; ++j) Ke[i * 24 + j] = Ke[j * 24 + i] = 0.5 * (Ke[i * 24 + j] + Ke[j * 24 + i]);
}

vfem_status prepareKe(const double* KeIn, KeData& k) {
    for (int i = 0; i < 576; ++i)
        if (!std::isfinite(KeIn[i])) return VFEM_ERR_INVALID_ARGUMENT;
    // Symmetrise from the upper triangle (src/FEM.cpp:200-210).
    for (int i = 0; i < 24; ++i) {
        k.Ke[i * 24 + i] = KeIn[i * 24 + i];
        for (int j = 0; j < i; ++j) k.Ke[i * 24 + j] = k.Ke[j * 24 + i] = KeIn[j * 24 + i];
        k.diag[i] = k.Ke[i * 24 + i];
    }
    // Walsh-Hadamard basis: H8[m][a] = prod_i (-1)^(m_i a_i); Khat = H Ke H^T / 64.
    auto h = [](int m, int a) { return (__builtin_popcount(m & a) & 1) ? -1.0 : 1.0; };
    double maxabs = 0;
    for (int i = 0; i < 24; ++i)
        for (int j = 0; j < 24; ++j) {
            int mi = i / 3, ci = i % 3, mj = j / 3, cj = j % 3;
            double s = 0;
            for (int a = 0; a < 8; ++a)
                for (int b = 0; b < 8; ++b) s += h(mi, a) * k.Ke[(3 * a + ci) * 24 + 3 * b + cj] * h(mj, b);
            k.Khat[i * 24 + j] = s / 64.0;
            maxabs = std::max(maxabs, std::fabs(s / 64.0));
        }
    bool onPat[576] = {};
    for (int p = 0; p < 45; ++p) {
        onPat[kPatRow[p] * 24 + kPatCol[p]] = true;
        k.ks[p] = k.Khat[kPatRow[p] * 24 + kPatCol[p]];
    }
    k.structured = true;
    for (int i = 0; i < 576; ++i)
        if (!onPat[i] && std::fabs(k.Khat[i]) > 1e-13 * maxabs) k.structured = false;
    return VFEM_OK;
}

namespace {
inline double tri1(int a, int b, int div) { return b == 0 ? double(div - a) / div : double(a) / div; }

}  // namespace

// Per-child diagonal of R_DOF^T (Ke at child ch) R_DOF (RestrictionOperator.hpp:246-708
// as the trilinear tensor product; child placement of RestrictionOperator.hpp:6-84).
void childDiagTable(const double* Ke, int div, std::vector<double>& tab) {
    int nch = div * div * div;
    tab.assign((size_t)nch * 24, 0.0);
    for (int ch = 0; ch < nch; ++ch) {
        int cx = ch % div, cy = (ch / div) % div, cz = ch / (div * div);
        for (int k = 0; k < 24; ++k) {
            int C = k / 3, c = k % 3;
            int bx = C & 1, by = (C >> 1) & 1, bz = (C >> 2) & 1;
            double r[8];
            for (int a = 0; a < 8; ++a) {
                int fx = cx + (a & 1), fy = cy + ((a >> 1) & 1), fz = cz + ((a >> 2) & 1);
                r[a] = tri1(fx, bx, div) * tri1(fy, by, div) * tri1(fz, bz, div);
            }
            double s = 0;
            for (int a = 0; a < 8; ++a)
                for (int b = 0; b < 8; ++b) s += r[a] * Ke[(3 * a + c) * 24 + 3 * b + c] * r[b];
            tab[(size_t)ch * 24 + k] = s;
        }
    }
}

void initGrid(Grid& g, int ex, int ey, int ez) {
    g.ex = ex; g.ey = ey; g.ez = ez;
    g.nx = ex + 1; g.ny = ey + 1; g.nz = ez + 1;
    g.nnode = (int64_t)g.nx * g.ny * g.nz;
}

vfem_status planLevels(int nx, int ny, int nz, int numLevels, int skip, std::vector<LevelPlan>& out,
                       std::string& err) {
    if (nx < 1 || ny < 1 || nz < 1 || numLevels < 1 || skip < 0 || skip > 1) {
        err = "invalid dimensions, level count or skip";
        return VFEM_ERR_INVALID_ARGUMENT;
    }
    if ((int64_t)(nx + 1) * (ny + 1) * (nz + 1) * 3 >= (int64_t)INT32_MAX) {
        err = "grid too large for 32-bit DOF indexing";
        return VFEM_ERR_INVALID_ARGUMENT;
    }
    out.clear();
    LevelPlan l0;
    initGrid(l0.g, nx, ny, nz);
    l0.div = 1;
    l0.scale = 1.0;
    out.push_back(l0);
    // Early stop once the (ceil-halved) reference dims reach <= 2 (FEM.cpp:465-470).
    int refDims[3] = {nx, ny, nz};
    for (int i = 1; i < numLevels; ++i) {
        const Grid& f = out.back().g;
        LevelPlan c;
        c.div = (i == 1 && skip > 0) ? (1 << (skip + 1)) : 2;
        initGrid(c.g, (f.ex + c.div - 1) / c.div, (f.ey + c.div - 1) / c.div, (f.ez + c.div - 1) / c.div);
        c.scale = std::pow(2.0, i + skip);
        out.push_back(c);
        for (int d = 0; d < 3; ++d) refDims[d] = refDims[d] / 2 + refDims[d] % 2;
        if (refDims[0] <= 2 || refDims[1] <= 2 || refDims[2] <= 2) break;
    }
    return VFEM_OK;
}

}  // namespace vfem
