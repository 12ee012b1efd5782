// setup_gpu.h -- device-side construction of the multigrid hierarchy (setup_gpu.cu).
#pragma once

#include <cuda_runtime.h>

#include "vfem_internal.h"

namespace vfem {

struct Diag24 {
    double v[24];  // diag(Ke)
};

// Device-side counters of one level's set-up (zero them before use).
struct SetupCounters {
    unsigned err;                 // level 0: bit 0 bad modulus on a filled voxel, bit 1 voxel value not 0/1
    unsigned pad;
    unsigned long long filled;    // level 0: filled voxels
    unsigned long long nelem;     // elements with a non-zero modulus
    long long nused;              // used nodes (after gpuCompactUsed)
};

// Level 0: modulus per element from the voxels (x fastest; Ein null = 1) and the
// used flag of every node.
cudaError_t gpuLevel0(cudaStream_t st, const Grid& g, const uint8_t* vox, const float* Ein, float* E, uint8_t* flags,
                      SetupCounters* cnt);

// nodeStore[k] = storage index of the k-th used node (increasing); cnt->nused.
// blockScratch holds compactScratchInts(g.nnode) ints.
cudaError_t gpuCompactUsed(cudaStream_t st, const Grid& g, const uint8_t* flags, int* blockScratch,
                           int32_t* nodeStore, SetupCounters* cnt);
int64_t compactScratchInts(int64_t nnode);

// flags[nodeStore[ids[i]]] |= FLAG_FIXED (ids validated by the caller).
cudaError_t gpuSetFixed(cudaStream_t st, int64_t n, const int64_t* ids, const int32_t* nodeStore, uint8_t* flags);

// Inverse diagonal of scale * sum_e E_e Ke (FP64 and FP32 copies, 3 per node).
cudaError_t gpuDiagRedisc(cudaStream_t st, const Grid& g, const float* E, const uint8_t* flags, double scale,
                          const Diag24& dg, double* d64, float* d32);

// A coarse level's moduli (mean of used children; volume average), used
// flags and dilated fixed flags.
cudaError_t gpuCoarseLevel(cudaStream_t st, const Grid& gf, const Grid& gc, int div, const float* Ef,
                           const float* Evf, const uint8_t* flagsF, float* Ec, float* Evc, uint8_t* flagsC,
                           SetupCounters* cnt);

// The reference's inverse diagonal of a coarse level (Galerkin for partial
// elements); tab = per-child diagonal table (div^3 x 24, device memory).
cudaError_t gpuDiagCoarse(cudaStream_t st, const Grid& gf, const Grid& gc, int div, const float* Ef, const float* Ec,
                          const uint8_t* flagsC, double scale, double childScale, const double* tab,
                          const Diag24& dg, double* d64, float* d32);

}  // namespace vfem
