// setup.cpp -- host-side set-up of the voxel multigrid hierarchy.
//
// Restates assembleSystemMatrix (src/FEM.cpp:157-517 of the reference) on dense
// structured grids instead of std::map node sets.  Every quantity the reference
// builds has a structured equivalent here:
//   * EnlistUsedElements + compressed numbering (FEM.cpp:66-100,179-186): a node
//     is used when a filled voxel touches it; compressed ids follow linear order,
//     which is the storage order of the dense node grid;
//   * coarse elements (FEM.cpp:274-283): a coarse element is used when any of its
//     children is used; dims are ceil-halved (ceil-quartered for the skipped
//     first level, FEM.cpp:266-272);
//   * restriction mapping + coefficients W = 1/multiplicity (FEM.cpp:340-362,400):
//     every coarse element whose bounding stencil holds fine node f also has as
//     corners all coarse nodes C with |f - d*C| < d, so the reference's
//     sum over elements of R[f,C] W[f] equals the plain trilinear weight of
//     (f - d*C); the kernels therefore apply full weighting with no tables;
//   * fixed nodes per level (FEM.cpp:402-460): restricting the 0/1 indicator and
//     keeping non-zeros is a dilation: C is fixed when any fixed fine node lies
//     within |f - d*C| < d;
//   * inverse diagonals (FEM.cpp:105-151,463): full coarse elements contribute
//     2^(l+skip) diag(Ke); partially filled ones contribute the diagonal of the
//     Galerkin matrix sum_children 2^(l-1) R^T Ke_child R (FEM.cpp:364-395),
//     accumulated child by child from a per-child table;
//   * early stop when the (ceil-halved) level dims reach <= 2 (FEM.cpp:465-470).
// Extension with no reference counterpart: a per-voxel modulus E.  Coarse
// elements carry the mean E of their used children; with E == 1 everything
// reduces to the reference.
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

// Per-child diagonal of R_DOF^T (Ke at child ch) R_DOF (RestrictionOperator.hpp:246-708
// as the trilinear tensor product; child placement of RestrictionOperator.hpp:6-84).
void childDiagTable(const double* Ke, int div, std::vector<double>& tab) {
    int nch = div * div * div, n = div + 1;
    tab.assign((size_t)nch * 24, 0.0);
    for (int ch = 0; ch < nch; ++ch) {
        int cx = ch % div, cy = (ch / div) % div, cz = ch / (div * div);
        for (int k = 0; k < 24; ++k) {
            int C = k / 3, c = k % 3;
            int bx = C & 1, by = (C >> 1) & 1, bz = (C >> 2) & 1;
            double r[8];
            for (int a = 0; a < 8; ++a) {
                int fx = cx + (a & 1), fy = cy + ((a >> 1) & 1), fz = cz + ((a >> 2) & 1);
                (void)n;
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

// Node flags from the element field; compressed numbering in storage order.
void markNodes(HostLevel& l) {
    const Grid& g = l.g;
    l.flags.assign(g.nnode, 0);
    l.nelem = 0;
    for (int z = 0; z < g.ez; ++z)
        for (int y = 0; y < g.ey; ++y)
            for (int x = 0; x < g.ex; ++x) {
                if (l.E[g.store(x, y, z)] == 0.f) continue;
                ++l.nelem;
                for (int d = 0; d < 8; ++d) l.flags[g.store(x + (d & 1), y + ((d >> 1) & 1), z + (d >> 2))] |= FLAG_USED;
            }
    l.nodeStore.clear();
    for (int64_t s = 0; s < g.nnode; ++s)
        if (l.flags[s] & FLAG_USED) l.nodeStore.push_back((int32_t)s);
}

void fixedIdsFromFlags(HostLevel& l) {
    l.fixedIds.clear();
    for (size_t i = 0; i < l.nodeStore.size(); ++i)
        if (l.flags[l.nodeStore[i]] & FLAG_FIXED) l.fixedIds.push_back((int64_t)i);
}

void invert(std::vector<double>& d, const std::vector<uint8_t>& flags) {
    for (size_t s = 0; s < flags.size(); ++s)
        for (int c = 0; c < 3; ++c) {
            double& v = d[3 * s + c];
            v = (flags[s] & FLAG_USED) ? 1.0 / v : 0.0;
        }
}

// Diagonal of scale * sum_e Ef_e Ke over the elements touching each node.
void rediscretisedDiag(const HostLevel& l, const std::vector<float>& Ef, const KeData& ke, std::vector<double>& d) {
    const Grid& g = l.g;
    d.assign(3 * g.nnode, 0.0);
    for (int z = 0; z < g.ez; ++z)
        for (int y = 0; y < g.ey; ++y)
            for (int x = 0; x < g.ex; ++x) {
                float E = Ef[g.store(x, y, z)];
                if (E == 0.f) continue;
                for (int a = 0; a < 8; ++a) {
                    int64_t s = g.store(x + (a & 1), y + ((a >> 1) & 1), z + (a >> 2));
                    for (int c = 0; c < 3; ++c) d[3 * s + c] += l.scale * (double)E * ke.diag[3 * a + c];
                }
            }
}

}  // namespace

vfem_status buildHierarchy(const uint8_t* vox, int nx, int ny, int nz, const float* Ein,
                           const int64_t* fixed, int64_t nfixed, int numLevels, int skip,
                           const KeData& ke, Hierarchy& H, std::string& err) {
    if (nx < 1 || ny < 1 || nz < 1 || numLevels < 1 || skip < 0 || skip > 1) {
        err = "invalid dimensions, level count or skip";
        return VFEM_ERR_INVALID_ARGUMENT;
    }
    if ((int64_t)(nx + 1) * (ny + 1) * (nz + 1) * 3 >= (int64_t)INT32_MAX) {
        err = "grid too large for 32-bit DOF indexing";
        return VFEM_ERR_INVALID_ARGUMENT;
    }
    H.L.clear();
    H.skip = skip;
    H.L.emplace_back();
    HostLevel& l0 = H.L[0];
    initGrid(l0.g, nx, ny, nz);
    l0.divider = 1;
    l0.scale = 1.0;
    l0.E.assign(l0.g.nnode, 0.f);
    int64_t filled = 0;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                int64_t v = ((int64_t)z * ny + y) * nx + x;
                if (vox[v] == 1) {
                    float e = Ein ? Ein[v] : 1.f;
                    if (!(e > 0.f) || !std::isfinite(e)) {
                        err = "non-positive or non-finite modulus on a filled voxel";
                        return VFEM_ERR_INVALID_ARGUMENT;
                    }
                    l0.E[l0.g.store(x, y, z)] = e;
                    ++filled;
                } else if (vox[v] != 0) {
                    err = "voxel values must be 0 or 1";
                    return VFEM_ERR_INVALID_ARGUMENT;
                }
            }
    if (filled == 0) {
        err = "no filled voxel";
        return VFEM_ERR_EMPTY;
    }
    markNodes(l0);
    int64_t nused = (int64_t)l0.nodeStore.size();
    for (int64_t i = 0; i < nfixed; ++i) {
        if (fixed[i] < 0 || fixed[i] >= nused) {
            err = "fixed node id out of range";
            return VFEM_ERR_INVALID_ARGUMENT;
        }
        l0.flags[l0.nodeStore[fixed[i]]] |= FLAG_FIXED;
    }
    fixedIdsFromFlags(l0);
    l0.Ev = l0.E;
    rediscretisedDiag(l0, l0.E, ke, l0.dinv);
    l0.dinvRedisc = l0.dinv;
    invert(l0.dinv, l0.flags);
    invert(l0.dinvRedisc, l0.flags);

    std::vector<double> tab2, tab4;
    childDiagTable(ke.Ke, 2, tab2);
    childDiagTable(ke.Ke, 4, tab4);
    int refDims[3] = {nx, ny, nz};
    for (int i = 1; i < numLevels; ++i) {
        const HostLevel& f = H.L[i - 1];
        int div = (i == 1 && skip > 0) ? (1 << (skip + 1)) : 2;
        HostLevel c;
        initGrid(c.g, (f.g.ex + div - 1) / div, (f.g.ey + div - 1) / div, (f.g.ez + div - 1) / div);
        c.divider = div;
        c.scale = std::pow(2.0, i + skip);
        int nch = div * div * div;
        const std::vector<double>& tab = div == 4 ? tab4 : tab2;
        double childScale = std::pow(2.0, i - 1);
        c.E.assign(c.g.nnode, 0.f);
        c.Ev.assign(c.g.nnode, 0.f);
        c.dinv.assign(3 * c.g.nnode, 0.0);
        // Coarse elements: used children, mean modulus, diagonal contributions.
        for (int z = 0; z < c.g.ez; ++z)
            for (int y = 0; y < c.g.ey; ++y)
                for (int x = 0; x < c.g.ex; ++x) {
                    double sumE = 0, sumEv = 0;
                    int cnt = 0;
                    double part[24] = {};
                    for (int ch = 0; ch < nch; ++ch) {
                        int fx = x * div + ch % div, fy = y * div + (ch / div) % div, fz = z * div + ch / (div * div);
                        if (fx >= f.g.ex || fy >= f.g.ey || fz >= f.g.ez) continue;
                        float Ef = f.E[f.g.store(fx, fy, fz)];
                        if (Ef == 0.f) continue;
                        ++cnt;
                        sumE += Ef;
                        sumEv += f.Ev[f.g.store(fx, fy, fz)];
                        for (int k = 0; k < 24; ++k) part[k] += childScale * (double)Ef * tab[(size_t)ch * 24 + k];
                    }
                    if (!cnt) continue;
                    float Ec = (float)(sumE / cnt);
                    c.E[c.g.store(x, y, z)] = Ec;
                    c.Ev[c.g.store(x, y, z)] = (float)(sumEv / nch);
                    bool full = cnt == nch;
                    for (int a = 0; a < 8; ++a) {
                        int64_t s = c.g.store(x + (a & 1), y + ((a >> 1) & 1), z + (a >> 2));
                        for (int cc = 0; cc < 3; ++cc) {
                            int k = 3 * a + cc;
                            c.dinv[3 * s + cc] += full ? c.scale * (double)Ec * ke.diag[k] : part[k];
                        }
                    }
                }
        markNodes(c);
        // Fixed dilation.
        int reach = div - 1;
        for (int z = 0; z < c.g.nz; ++z)
            for (int y = 0; y < c.g.ny; ++y)
                for (int x = 0; x < c.g.nx; ++x) {
                    bool fx_ = false;
                    for (int dz = -reach; dz <= reach && !fx_; ++dz)
                        for (int dy = -reach; dy <= reach && !fx_; ++dy)
                            for (int dx = -reach; dx <= reach && !fx_; ++dx) {
                                int X = x * div + dx, Y = y * div + dy, Z = z * div + dz;
                                if (X < 0 || Y < 0 || Z < 0 || X >= f.g.nx || Y >= f.g.ny || Z >= f.g.nz) continue;
                                if (f.flags[f.g.store(X, Y, Z)] & FLAG_FIXED) fx_ = true;
                            }
                    if (fx_) c.flags[c.g.store(x, y, z)] |= FLAG_FIXED;
                }
        fixedIdsFromFlags(c);
        rediscretisedDiag(c, c.Ev, ke, c.dinvRedisc);
        invert(c.dinv, c.flags);
        invert(c.dinvRedisc, c.flags);
        H.L.push_back(std::move(c));
        for (int d = 0; d < 3; ++d) refDims[d] = refDims[d] / 2 + refDims[d] % 2;
        if (refDims[0] <= 2 || refDims[1] <= 2 || refDims[2] <= 2) break;
    }
    // Coarsest free DOFs (FEM.cpp:473-496), in compressed (storage) order.
    const HostLevel& lc = H.L.back();
    H.coarseFreeDof.clear();
    H.coarseFreeNode.assign(lc.g.nnode, -1);
    int32_t nf = 0;
    for (int32_t s : lc.nodeStore) {
        if (lc.flags[s] & FLAG_FIXED) continue;
        H.coarseFreeNode[s] = nf++;
        for (int cc = 0; cc < 3; ++cc) H.coarseFreeDof.push_back(3 * s + cc);
    }
    return VFEM_OK;
}

}  // namespace vfem
