// reduce.cuh -- device helpers shared by the kernel translation units: the
// deterministic block + grid reduction, the solver-scalar epilogues and the
// mixed-precision residual-replacement test.  Everything here has internal
// linkage (one copy per translation unit).
#pragma once

#include <cfloat>

#include "kernels.h"

namespace vfem {
namespace {

__device__ __forceinline__ double warpSum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Deterministic block + grid reduction of K sums.  Returns true in thread 0 of
// the last block to finish, with the totals in tot.  NTH = threads per block.
template <int NTH, int K>
__device__ __forceinline__ bool gridReduce(double (&v)[K], const RedBuf& rb, double (&tot)[K]) {
    static_assert(K >= 1 && K <= kMaxRedTerms, "more sums than the partials buffer holds");
    __shared__ double sred[K][NTH / 32];
    __shared__ int amLast;
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int lane = tid & 31, warp = tid >> 5;
    const unsigned nb = gridDim.x * gridDim.y * gridDim.z;
    const unsigned bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double s = warpSum(v[k]);
        if (lane == 0) sred[k][warp] = s;
    }
    __syncthreads();
    if (tid == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double s = 0;
            for (int w = 0; w < NTH / 32; ++w) s += sred[k][w];
            rb.partials[(size_t)k * kMaxRedBlocks + bid] = s;
        }
        __threadfence();
        unsigned t = atomicAdd(rb.ticket, 1u);
        amLast = (t == nb - 1);
    }
    __syncthreads();
    if (!amLast) return false;
    __threadfence();
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double s = 0;
        for (unsigned i = tid; i < nb; i += NTH) s += __ldcg(&rb.partials[(size_t)k * kMaxRedBlocks + i]);
        s = warpSum(s);
        if (lane == 0) sred[k][warp] = s;
    }
    __syncthreads();
    if (tid == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double s = 0;
            for (int w = 0; w < NTH / 32; ++w) s += sred[k][w];
            tot[k] = s;
        }
        *rb.ticket = 0u;
    }
    return tid == 0;
}

__device__ void applyEpi(int epi, Scalars* S, double t0, double t1) {
    switch (epi) {
        case EPI_STORE:
            S->red0 = t0;
            S->red1 = t1;
            break;
        case EPI_ALPHA:
            if (S->breakAt > 0 && S->iter + 1 >= S->breakAt) t0 = -1.0;  // forced breakdown (testing)
            S->pAp = t0;
            S->matvecs++;
            if (!(t0 > 0.0) || !isfinite(t0)) S->done = BREAKDOWN;
            else S->alpha = S->rho / t0;
            break;
        case EPI_CONV:
            S->rr = t0;
            S->rStamp = S->matvecs;
            if (!isfinite(t0)) S->done = BREAKDOWN;
            else if (t0 < S->threshold) {
                if (S->mixed) S->checkPending = 1;
                else S->done = CONVERGED;
            }
            break;
        case EPI_RHO0:
            S->rho = t0;
            if (!isfinite(t0)) S->done = BREAKDOWN;
            break;
        case EPI_BETA:
            S->rhoOld = S->rho;
            S->rho = t0;
            S->zAp = t1;
            S->beta = S->flexible ? -t1 / S->pAp : t0 / S->rhoOld;
            S->iter++;
            if (!isfinite(S->beta)) S->done = BREAKDOWN;
            else if (S->iter >= S->maxIter) S->done = MAXITER;
            break;
        case EPI_INIT:
            S->rhsNorm2 = t0;
            S->rr = t1;
            S->rrLast = t1;
            S->threshold = fmax(S->tol2 * t0, DBL_MIN);
            if (t0 == 0.0 || t1 < S->threshold) S->done = CONVERGED;
            break;
        case EPI_TRUE:
            if (S->replacements > 0 && t0 >= 0.98 * S->rrTruePrev) S->stalls++;
            else S->stalls = 0;
            S->rrTruePrev = t0;
            S->replStamp = S->matvecs;
            S->rrTrue = t0;
            S->rr = t0;
            S->rrLast = t0;
            S->checkPending = 0;
            S->replacements++;
            if (!isfinite(t0)) S->done = BREAKDOWN;
            else if (t0 < S->threshold) S->done = CONVERGED;
            else if (S->stalls >= 3) S->done = STAGNATED;
            break;
        default:
            break;
    }
}

// Mixed precision: the FP64 true residual replaces the FP32 recursive one when
// the recursive residual claims convergence, every replaceEvery iterations, and
// whenever it has dropped by delta since the last replacement (the reliable-
// update rule of Sleijpen & van der Vorst, which keeps the FP32 drift small
// relative to the residual being replaced).
__device__ __forceinline__ bool trueResidualDue(const Scalars* S) {
    return S->checkPending || (S->replaceEvery > 0 && S->iter > 0 && (S->iter % S->replaceEvery) == 0) ||
           (S->delta2 > 0.0 && S->rr < S->delta2 * S->rrLast);
}

// Per-thread dot-product accumulator.  FP64 vectors accumulate in FP64.  FP32
// vectors accumulate in FP32 with Kahan compensation and are converted to FP64
// once per thread, before the FP64 block and grid reduction: on GB300 the FP64
// pipe is ~1/64 of FP32, so per-element FP64 conversions and FMAs would bound
// the FP32 kernels.
template <typename T>
struct DotAcc;
template <>
struct DotAcc<double> {
    double s = 0.0;
    __device__ __forceinline__ void add(double v) { s += v; }
    __device__ __forceinline__ double get() const { return s; }
};
template <>
struct DotAcc<float> {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float v) {
        const float y = v - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double get() const { return (double)s - (double)c; }
};

}  // namespace
}  // namespace vfem
