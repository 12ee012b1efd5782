// setup_gpu.cu -- the multigrid hierarchy built on the device.
//
// Restates assembleSystemMatrix (src/FEM.cpp:157-517 of the reference) on dense
// structured grids, one data-parallel kernel per step, instead of std::map node
// sets walked on the host.  Every quantity the reference builds has a structured
// equivalent:
//   * EnlistUsedElements + compressed numbering (FEM.cpp:66-100,179-186): a node
//     is used when a filled voxel touches it; compressed ids follow linear order,
//     which is the storage order of the dense node grid (a stream compaction);
//   * coarse elements (FEM.cpp:274-283): a coarse element is used when any of its
//     children is used; dims are ceil-halved (ceil-quartered for the skipped
//     first level, FEM.cpp:266-272);
//   * restriction mapping + coefficients W = 1/multiplicity (FEM.cpp:340-362,400):
//     every coarse element whose bounding stencil holds fine node f also has as
//     corners all coarse nodes C with |f - d*C| < d, so the reference's sum over
//     elements of R[f,C] W[f] equals the plain trilinear weight of (f - d*C); the
//     transfer kernels therefore apply full weighting with no tables;
//   * fixed nodes per level (FEM.cpp:402-460): restricting the 0/1 indicator and
//     keeping non-zeros is a dilation: C is fixed when any fixed fine node lies
//     within |f - d*C| < d;
//   * inverse diagonals (FEM.cpp:105-151,463): full coarse elements contribute
//     2^(l+skip) diag(Ke); partially filled ones contribute the diagonal of the
//     Galerkin matrix sum_children 2^(l-1) R^T Ke_child R (FEM.cpp:364-395),
//     accumulated child by child from a per-child table (setup.cpp).
// Extension with no reference counterpart: a per-voxel modulus E.  Coarse
// elements carry the mean E of their used children; with E == 1 everything
// reduces to the reference.  Every kernel gathers (one thread per output), so
// no floating-point atomics are used and the result does not depend on
// scheduling.
#include "setup_gpu.h"

namespace vfem {

namespace {

constexpr int NT = 256;

inline unsigned flatGrid(int64_t n) {
    int64_t b = (n + NT - 1) / NT;
    if (b > 152 * 16) b = 152 * 16;
    return (unsigned)(b < 1 ? 1 : b);
}

// Level 0: modulus per element (lower-corner storage index) from the voxels
// (x fastest).  err |= 1: non-positive or non-finite modulus on a filled voxel;
// err |= 2: a voxel value other than 0 or 1.  filled counts the filled voxels.
__global__ void kVoxelsToE(Grid g, const uint8_t* __restrict__ vox, const float* __restrict__ Ein,
                           float* __restrict__ E, unsigned* err, unsigned long long* filled) {
    const int64_t nv = (int64_t)g.ex * g.ey * g.ez;
    unsigned long long cnt = 0;
    unsigned bad = 0;
    for (int64_t v = blockIdx.x * (int64_t)NT + threadIdx.x; v < nv; v += (int64_t)gridDim.x * NT) {
        const int x = (int)(v % g.ex), y = (int)((v / g.ex) % g.ey), z = (int)(v / ((int64_t)g.ex * g.ey));
        const uint8_t b = vox[v];
        float e = 0.f;
        if (b == 1) {
            e = Ein ? Ein[v] : 1.f;
            if (!(e > 0.f) || !isfinite(e)) bad |= 1u;
            ++cnt;
        } else if (b != 0) {
            bad |= 2u;
        }
        E[g.store(x, y, z)] = e;
    }
    if (bad) atomicOr(err, bad);
    if (cnt) atomicAdd(filled, cnt);
}

// Used flag of every node (a filled element touches it); nelem counts elements.
__global__ void kMarkUsed(Grid g, const float* __restrict__ E, uint8_t* __restrict__ flags,
                          unsigned long long* nelem) {
    unsigned long long cnt = 0;
    for (int64_t s = blockIdx.x * (int64_t)NT + threadIdx.x; s < g.nnode; s += (int64_t)gridDim.x * NT) {
        const int x = (int)(s % g.nx), y = (int)((s / g.nx) % g.ny), z = (int)(s / ((int64_t)g.nx * g.ny));
        bool used = false;
#pragma unroll
        for (int a = 0; a < 8; ++a) {
            const int ex = x - (a & 1), ey = y - ((a >> 1) & 1), ez = z - (a >> 2);
            if (ex >= 0 && ey >= 0 && ez >= 0 && ex < g.ex && ey < g.ey && ez < g.ez && E[g.store(ex, ey, ez)] != 0.f)
                used = true;
        }
        flags[s] = used ? FLAG_USED : 0;
        if (x < g.ex && y < g.ey && z < g.ez && E[s] != 0.f) ++cnt;
    }
    if (cnt) atomicAdd(nelem, cnt);
}

// ---- stream compaction of the used nodes, in storage order.
// A block owns kChunk consecutive nodes; pass 1 counts, pass 2 scans the block
// counts, pass 3 writes each used node at its block offset plus its rank.
constexpr int kChunk = 16 * NT;

__global__ void kCountUsed(int64_t n, const uint8_t* __restrict__ flags, int* __restrict__ blockCount) {
    __shared__ int ws[NT / 32];
    const int64_t base = blockIdx.x * (int64_t)kChunk;
    int c = 0;
    for (int r = 0; r < kChunk / NT; ++r) {
        const int64_t s = base + r * NT + threadIdx.x;
        c += (s < n && (flags[s] & FLAG_USED)) ? 1 : 0;
    }
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < NT / 32; ++w) t += ws[w];
        blockCount[blockIdx.x] = t;
    }
}

// Exclusive scan of nb block counts in place, total into *total (one block).
__global__ void kScanCounts(int nb, int* __restrict__ counts, long long* total) {
    __shared__ int ws[1024 / 32];
    __shared__ long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int base = 0; base < nb; base += 1024) {
        const int i = base + threadIdx.x;
        const int v = i < nb ? counts[i] : 0;
        int incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) ws[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            int w = ws[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += t;
            }
            ws[lane] = w;  // inclusive scan of warp sums
        }
        __syncthreads();
        const long long excl = carry + (warp ? ws[warp - 1] : 0) + incl - v;
        if (i < nb) counts[i] = (int)excl;
        __syncthreads();
        if (threadIdx.x == 1023) carry = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void kWriteUsed(int64_t n, const uint8_t* __restrict__ flags, const int* __restrict__ blockOffset,
                           int32_t* __restrict__ nodeStore) {
    __shared__ int ws[NT / 32];
    __shared__ int running;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) running = blockOffset[blockIdx.x];
    __syncthreads();
    const int64_t base = blockIdx.x * (int64_t)kChunk;
    for (int r = 0; r < kChunk / NT; ++r) {
        const int64_t s = base + r * NT + threadIdx.x;
        const bool u = s < n && (flags[s] & FLAG_USED);
        const unsigned m = __ballot_sync(0xffffffffu, u);
        if (lane == 0) ws[warp] = __popc(m);
        __syncthreads();
        int before = running;
        for (int w = 0; w < warp; ++w) before += ws[w];
        if (u) nodeStore[before + __popc(m & ((1u << lane) - 1u))] = (int32_t)s;
        __syncthreads();
        if (threadIdx.x == 0) {
            int t = 0;
            for (int w = 0; w < NT / 32; ++w) t += ws[w];
            running += t;
        }
        __syncthreads();
    }
}

__global__ void kSetFixed(int64_t n, const int64_t* __restrict__ ids, const int32_t* __restrict__ nodeStore,
                          uint8_t* __restrict__ flags) {
    for (int64_t i = blockIdx.x * (int64_t)NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT)
        flags[nodeStore[ids[i]]] |= FLAG_FIXED;
}

// Inverse of the diagonal of scale * sum_e Ee Ke over the elements touching each
// node (0 at unused nodes): the fine level's reference diagonal and every
// level's rediscretised one.
__global__ void kDiagRedisc(Grid g, const float* __restrict__ E, const uint8_t* __restrict__ flags, double scale,
                            Diag24 dg, double* __restrict__ d64, float* __restrict__ d32) {
    for (int64_t s = blockIdx.x * (int64_t)NT + threadIdx.x; s < g.nnode; s += (int64_t)gridDim.x * NT) {
        const int x = (int)(s % g.nx), y = (int)((s / g.nx) % g.ny), z = (int)(s / ((int64_t)g.nx * g.ny));
        double d[3] = {0.0, 0.0, 0.0};
        // elements in increasing storage order; the node is corner a of element (x,y,z) - offset(a)
#pragma unroll
        for (int a = 7; a >= 0; --a) {
            const int ex = x - (a & 1), ey = y - ((a >> 1) & 1), ez = z - (a >> 2);
            if (ex < 0 || ey < 0 || ez < 0 || ex >= g.ex || ey >= g.ey || ez >= g.ez) continue;
            const float e = E[g.store(ex, ey, ez)];
            if (e == 0.f) continue;
#pragma unroll
            for (int c = 0; c < 3; ++c) d[c] += scale * (double)e * dg.v[3 * a + c];
        }
        const bool used = flags[s] & FLAG_USED;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double inv = used ? 1.0 / d[c] : 0.0;
            d64[3 * s + c] = inv;
            d32[3 * s + c] = (float)inv;
        }
    }
}

// Coarse element moduli: E = mean over used children, Ev = sum over children / div^3.
__global__ void kCoarsenE(Grid gf, Grid gc, int div, const float* __restrict__ Ef, const float* __restrict__ Evf,
                          float* __restrict__ Ec, float* __restrict__ Evc) {
    const int nch = div * div * div;
    for (int64_t s = blockIdx.x * (int64_t)NT + threadIdx.x; s < gc.nnode; s += (int64_t)gridDim.x * NT) {
        const int x = (int)(s % gc.nx), y = (int)((s / gc.nx) % gc.ny), z = (int)(s / ((int64_t)gc.nx * gc.ny));
        float e = 0.f, ev = 0.f;
        if (x < gc.ex && y < gc.ey && z < gc.ez) {
            double sumE = 0, sumEv = 0;
            int cnt = 0;
            for (int ch = 0; ch < nch; ++ch) {
                const int fx = x * div + ch % div, fy = y * div + (ch / div) % div, fz = z * div + ch / (div * div);
                if (fx >= gf.ex || fy >= gf.ey || fz >= gf.ez) continue;
                const float v = Ef[gf.store(fx, fy, fz)];
                if (v == 0.f) continue;
                ++cnt;
                sumE += v;
                sumEv += Evf[gf.store(fx, fy, fz)];
            }
            if (cnt) {
                e = (float)(sumE / cnt);
                ev = (float)(sumEv / nch);
            }
        }
        Ec[s] = e;
        Evc[s] = ev;
    }
}

// Coarse fixed flags: C is fixed when a fixed fine node lies within |f - div*C| < div.
__global__ void kFixedDilate(Grid gf, Grid gc, int div, const uint8_t* __restrict__ ff, uint8_t* __restrict__ fc) {
    const int reach = div - 1;
    for (int64_t s = blockIdx.x * (int64_t)NT + threadIdx.x; s < gc.nnode; s += (int64_t)gridDim.x * NT) {
        const int x = (int)(s % gc.nx), y = (int)((s / gc.nx) % gc.ny), z = (int)(s / ((int64_t)gc.nx * gc.ny));
        bool fixed = false;
        for (int dz = -reach; dz <= reach && !fixed; ++dz)
            for (int dy = -reach; dy <= reach && !fixed; ++dy)
                for (int dx = -reach; dx <= reach && !fixed; ++dx) {
                    const int X = x * div + dx, Y = y * div + dy, Z = z * div + dz;
                    if (X < 0 || Y < 0 || Z < 0 || X >= gf.nx || Y >= gf.ny || Z >= gf.nz) continue;
                    if (ff[gf.store(X, Y, Z)] & FLAG_FIXED) fixed = true;
                }
        if (fixed) fc[s] |= FLAG_FIXED;
    }
}

// Reference inverse diagonal of a coarse level: per coarse node, over its coarse
// elements: full elements (all div^3 children inside the fine grid and used)
// add scale * Ec * diag(Ke); partial ones add the Galerkin child diagonals
// childScale * Ef * tab[child] of their used children.
__global__ void kDiagCoarse(Grid gf, Grid gc, int div, const float* __restrict__ Ef, const float* __restrict__ Ec,
                            const uint8_t* __restrict__ flags, double scale, double childScale,
                            const double* __restrict__ tab, Diag24 dg, double* __restrict__ d64,
                            float* __restrict__ d32) {
    const int nch = div * div * div;
    for (int64_t s = blockIdx.x * (int64_t)NT + threadIdx.x; s < gc.nnode; s += (int64_t)gridDim.x * NT) {
        const int x = (int)(s % gc.nx), y = (int)((s / gc.nx) % gc.ny), z = (int)(s / ((int64_t)gc.nx * gc.ny));
        double d[3] = {0.0, 0.0, 0.0};
        for (int a = 7; a >= 0; --a) {
            const int ex = x - (a & 1), ey = y - ((a >> 1) & 1), ez = z - (a >> 2);
            if (ex < 0 || ey < 0 || ez < 0 || ex >= gc.ex || ey >= gc.ey || ez >= gc.ez) continue;
            const float e = Ec[gc.store(ex, ey, ez)];
            if (e == 0.f) continue;
            double part[3] = {0.0, 0.0, 0.0};
            int cnt = 0;
            for (int ch = 0; ch < nch; ++ch) {
                const int fx = ex * div + ch % div, fy = ey * div + (ch / div) % div, fz = ez * div + ch / (div * div);
                if (fx >= gf.ex || fy >= gf.ey || fz >= gf.ez) continue;
                const float v = Ef[gf.store(fx, fy, fz)];
                if (v == 0.f) continue;
                ++cnt;
                for (int c = 0; c < 3; ++c) part[c] += childScale * (double)v * tab[ch * 24 + 3 * a + c];
            }
            for (int c = 0; c < 3; ++c) d[c] += cnt == nch ? scale * (double)e * dg.v[3 * a + c] : part[c];
        }
        const bool used = flags[s] & FLAG_USED;
        for (int c = 0; c < 3; ++c) {
            const double inv = used ? 1.0 / d[c] : 0.0;
            d64[3 * s + c] = inv;
            d32[3 * s + c] = (float)inv;
        }
    }
}

}  // namespace

cudaError_t gpuLevel0(cudaStream_t st, const Grid& g, const uint8_t* vox, const float* Ein, float* E, uint8_t* flags,
                      SetupCounters* cnt) {
    cudaError_t e = cudaMemsetAsync(E, 0, sizeof(float) * (size_t)g.nnode, st);
    if (e != cudaSuccess) return e;
    kVoxelsToE<<<flatGrid((int64_t)g.ex * g.ey * g.ez), NT, 0, st>>>(g, vox, Ein, E, &cnt->err, &cnt->filled);
    kMarkUsed<<<flatGrid(g.nnode), NT, 0, st>>>(g, E, flags, &cnt->nelem);
    return cudaGetLastError();
}

cudaError_t gpuCompactUsed(cudaStream_t st, const Grid& g, const uint8_t* flags, int* blockScratch,
                           int32_t* nodeStore, SetupCounters* cnt) {
    const int64_t nb = (g.nnode + kChunk - 1) / kChunk;
    kCountUsed<<<(unsigned)nb, NT, 0, st>>>(g.nnode, flags, blockScratch);
    kScanCounts<<<1, 1024, 0, st>>>((int)nb, blockScratch, &cnt->nused);
    kWriteUsed<<<(unsigned)nb, NT, 0, st>>>(g.nnode, flags, blockScratch, nodeStore);
    return cudaGetLastError();
}

int64_t compactScratchInts(int64_t nnode) { return (nnode + kChunk - 1) / kChunk; }

cudaError_t gpuSetFixed(cudaStream_t st, int64_t n, const int64_t* ids, const int32_t* nodeStore, uint8_t* flags) {
    if (n > 0) kSetFixed<<<flatGrid(n), NT, 0, st>>>(n, ids, nodeStore, flags);
    return cudaGetLastError();
}

cudaError_t gpuDiagRedisc(cudaStream_t st, const Grid& g, const float* E, const uint8_t* flags, double scale,
                          const Diag24& dg, double* d64, float* d32) {
    kDiagRedisc<<<flatGrid(g.nnode), NT, 0, st>>>(g, E, flags, scale, dg, d64, d32);
    return cudaGetLastError();
}

cudaError_t gpuCoarseLevel(cudaStream_t st, const Grid& gf, const Grid& gc, int div, const float* Ef,
                           const float* Evf, const uint8_t* flagsF, float* Ec, float* Evc, uint8_t* flagsC,
                           SetupCounters* cnt) {
    kCoarsenE<<<flatGrid(gc.nnode), NT, 0, st>>>(gf, gc, div, Ef, Evf, Ec, Evc);
    kMarkUsed<<<flatGrid(gc.nnode), NT, 0, st>>>(gc, Ec, flagsC, &cnt->nelem);
    kFixedDilate<<<flatGrid(gc.nnode), NT, 0, st>>>(gf, gc, div, flagsF, flagsC);
    return cudaGetLastError();
}

cudaError_t gpuDiagCoarse(cudaStream_t st, const Grid& gf, const Grid& gc, int div, const float* Ef, const float* Ec,
                          const uint8_t* flagsC, double scale, double childScale, const double* tab,
                          const Diag24& dg, double* d64, float* d32) {
    kDiagCoarse<<<flatGrid(gc.nnode), NT, 0, st>>>(gf, gc, div, Ef, Ec, flagsC, scale, childScale, tab, dg, d64, d32);
    return cudaGetLastError();
}

}  // namespace vfem
