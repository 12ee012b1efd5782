// api.cu -- problem lifecycle, the device-resident PCG driver and the C ABI.
//
// Replaces solveWithKompute (src/FEMGPU.cpp:32-554 of the reference) and the
// Eigen CG driver solveWithEigen (src/FEM.cpp:589-637).  The reference's GPU
// loop uploads and downloads full vectors and solves the coarsest level on the
// host every iteration (FEMGPU.cpp:471-541); here every step of an iteration
// is a kernel on one stream, the coarsest solve is a dense inverse applied on
// the device, and chunks of iterations are replayed as one CUDA graph with the
// host polling a device-side `done` flag between chunks.  The iteration count
// and stopping rule are Eigen 3.4's (x0 = 0, stop when |r|^2 < tol^2 |b|^2 on the
// recursive residual, iterations counted without the breaking pass).
#include <cuda_runtime.h>
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstddef>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <thread>
#include <type_traits>
#include <vector>

#include "kernels.h"
#include "setup_gpu.h"

using namespace vfem;

namespace {

std::atomic<long long> g_launches{0};
thread_local std::string g_lastError;

// Dense coarsest inverse.  Peak device memory while it is built, at the limit
// n = 65,536: the mixed solver's FP32 matrix (17.2 GB), the syrk result of the
// 64-bit path (another 17.2 GB) and the FP16 tiles (8.6 GB), about 43 GB; an
// FP64 inverse on that path needs 34.4 GB for the matrix plus 34.4 GB for the
// syrk result (the FP32 one's memory is released by then, its FP16 tiles stay).
constexpr int64_t kMaxCoarseFree = 65536;
constexpr int64_t kMaxCoarse32 = 32768;    // above: the 64-bit cuSOLVER path (n^2 >= 2^31)

// Testing hooks, read from the environment when a problem is created:
//   VFEM_COARSE_64BIT_MIN=n   coarsest systems with more than n free DOFs take
//                             the 64-bit factorisation path (default 32768);
//   VFEM_FAULT_ALLOC_AT=k     the k-th device allocation of the set-up (1-based)
//                             fails as if the device were out of memory.
thread_local int64_t g_coarse64Min = kMaxCoarse32;
thread_local long long g_allocCountdown = 0;
long long envInt(const char* name, long long dflt) {
    const char* v = std::getenv(name);
    if (!v || !*v) return dflt;
    char* end = nullptr;
    const long long x = std::strtoll(v, &end, 10);
    return (end && *end == 0) ? x : dflt;
}

struct DevLevel {
    Grid g;
    int div = 2;
    double scale = 1.0;
    int64_t nused = 0, nelem = 0;
    float* E = nullptr;
    float* Ev = nullptr;  // multiplicative-cycle modulus (volume average; aliases E on the finest level)
    uint8_t* flags = nullptr;
    int32_t* nodeStore = nullptr;
    double* dinv64 = nullptr;
    float* dinv32 = nullptr;
    double* dinvR64 = nullptr;
    float* dinvR32 = nullptr;
    // The reference cycle's inverse diagonal for the mixed V-cycle: FP16 values
    // times dinvHScale (a power of two mapping the largest entry into (2^13, 2^14]).
    __half* dinvH = nullptr;
    float dinvHScale = 1.0f;
    double *r64 = nullptr, *z64 = nullptr, *t64 = nullptr;
    float *r32 = nullptr, *z32 = nullptr, *t32 = nullptr;
    int64_t nvec() const { return 3 * g.nnode; }
};

struct GraphKey {
    int mg, prec, flexible, pre, post, replace, chunk;
    double omega;
    int parity;  // which buffer holds the level-0 residual when the chunk starts
    bool operator<(const GraphKey& o) const {
        return std::tie(mg, prec, flexible, pre, post, replace, chunk, omega, parity) <
               std::tie(o.mg, o.prec, o.flexible, o.pre, o.post, o.replace, o.chunk, o.omega, o.parity);
    }
};

struct CachedGraph {
    cudaGraphExec_t exec = nullptr;
    long long kernels = 0;
};

}  // namespace

struct vfem_problem {
    int device = 0;
    cudaStream_t stream = nullptr;
    KeData ke;
    std::vector<DevLevel> L;
    // coarsest level (built from its device flags at set-up)
    std::vector<int32_t> coarseFreeDof;   // storage DOF index (3*s + c) of each free coarse DOF
    std::vector<int32_t> coarseFreeNode;  // storage node -> free node id, -1 otherwise
    // level-0 solver vectors (dense storage)
    double *f64 = nullptr, *x64 = nullptr, *p64 = nullptr, *Ap64 = nullptr;
    float *p32 = nullptr, *Ap32 = nullptr;
    float* x32 = nullptr;  // mixed precision: FP32 solution correction since the last FP64 flush
    float* r32b = nullptr;  // mixed precision: the level-0 residual alternates between L[0].r32 and this
    float* p32b = nullptr;  // fused direction update: the FP32 direction alternates between p32 and this
    // coarsest dense inverse
    int64_t nc = 0;
    int32_t* freeDof = nullptr;
    // Coarsest dense inverses, built on first use (ensureCoarse): FP64 (full
    // n x n) for the FP64 solver and preconditioner; for the mixed one the FP32
    // inverse packed as the lower block triangle of 64 x 64 FP16 tiles
    // (launchPackSymHalf) with its power-of-two scale; V = the multiplicative
    // cycle's operator (volume-averaged modulus).
    double* Kinv64 = nullptr;
    double* KinvV64 = nullptr;
    __half* KinvH = nullptr;
    __half* KinvVH = nullptr;
    float scaleH = 1.0f, scaleVH = 1.0f;
    int32_t* dFreeNode = nullptr;  // coarsest storage node -> free node id (assembly)
    double* cb64 = nullptr;        // gathered coarse right-hand side, coarseBlocks(nc) * 64 (zero tail)
    float* cb32 = nullptr;
    double* cpart = nullptr;       // per-tile partial products, 128 per tile (used as float or double)
    // reductions / scalars
    Scalars* S = nullptr;
    Scalars* hS = nullptr;
    RedBuf rb{};
    // compressed staging (measured on GB300: kernels reading and writing the
    // caller's pageable host arrays directly were slower than these copies)
    unsigned* dFlag = nullptr;  // non-finite input flag of the scatter
    double* dComp = nullptr;  // 3 * nused(level 0) (largest level)
    double* hIn = nullptr;    // pinned
    double* hOut = nullptr;   // pinned
    // constants for the kernels
    double op64[45 + 576];
    float op32[45 + 576];
    // the tensor-core FP32 CG product (matvec_tc.cu), opt-in, when Ke admits an exact BF16 scaling
    TcOperand tc;
    bool tcReady = false;
    int tma = 0;  // bit 0: TMA-staged FP32 restrictions, bit 1: bulk-staged mixed prolongation (LaunchCtx::tma)
    bool pxFused = false;  // mixed solve: direction update fused into the CG product (launchMatvecPX)
    // deflation coarse space (vfem_problem_set_coarse_space): k dense columns V and K V
    int coarseK = 0, coarseCap = 0;
    double* V64 = nullptr;
    float* V32 = nullptr;
    double* KV64 = nullptr;
    float* KV32 = nullptr;
    CoarseSpace coarseG{};
    std::map<GraphKey, CachedGraph> graphs;
    bool rhsSet = false;
    long long launches = 0;
};

namespace {

vfem_status fail(vfem_status s, const std::string& msg) {
    g_lastError = msg;
    return s;
}

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) {                                                                   \
            return fail(e_ == cudaErrorMemoryAllocation ? VFEM_ERR_OUT_OF_MEMORY : VFEM_ERR_CUDA,  \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                       \
        }                                                                                          \
    } while (0)

// Zeroed device allocation.  The memset runs on the legacy default stream, which
// the problem's non-blocking stream does not wait for, so it is completed here:
// otherwise a set-up kernel could see the previous owner's bytes of a recycled
// block (a stale error flag, for example).
template <typename T>
cudaError_t dalloc(T** p, int64_t n) {
    if (g_allocCountdown > 0 && --g_allocCountdown == 0) return cudaErrorMemoryAllocation;  // testing hook
    // 64 spare zero bytes: bulk copies widen their ranges to 16-byte boundaries
    const size_t bytes = (size_t)std::max<int64_t>(n, 1) * sizeof(T) + 64;
    cudaError_t e = cudaMalloc((void**)p, bytes);
    if (e != cudaSuccess) return e;
    e = cudaMemset(*p, 0, bytes);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(cudaStreamLegacy);
}

// Device copy of a host vector, complete on return (a pageable cudaMemcpy may
// return before its DMA has landed).
template <typename T>
cudaError_t upload(T** p, const std::vector<T>& v) {
    cudaError_t e = dalloc(p, (int64_t)v.size());
    if (e != cudaSuccess || v.empty()) return e;
    e = cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(cudaStreamLegacy);
}

void freeProblem(vfem_problem* p) {
    if (!p) return;
    cudaSetDevice(p->device);
    for (auto& kv : p->graphs)
        if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    for (auto& l : p->L) {
        if (l.Ev != l.E) cudaFree(l.Ev);
        cudaFree(l.E); cudaFree(l.flags); cudaFree(l.nodeStore);
        cudaFree(l.dinv64); cudaFree(l.dinv32); cudaFree(l.dinvR64); cudaFree(l.dinvR32); cudaFree(l.dinvH);
        cudaFree(l.r64); cudaFree(l.z64); cudaFree(l.t64); cudaFree(l.r32); cudaFree(l.z32); cudaFree(l.t32);
    }
    cudaFree(p->f64); cudaFree(p->x64); cudaFree(p->p64); cudaFree(p->Ap64); cudaFree(p->p32); cudaFree(p->Ap32);
    cudaFree(p->x32); cudaFree(p->r32b); cudaFree(p->p32b);
    cudaFree(p->freeDof); cudaFree(p->Kinv64); cudaFree(p->KinvH); cudaFree(p->cb64); cudaFree(p->cb32);
    cudaFree(p->KinvV64); cudaFree(p->KinvVH); cudaFree(p->dFreeNode); cudaFree(p->cpart);
    cudaFree(p->dFlag); cudaFree(p->V64); cudaFree(p->V32); cudaFree(p->KV64); cudaFree(p->KV32);
    cudaFree(p->S); cudaFree(p->rb.partials); cudaFree(p->rb.ticket); cudaFree(p->dComp);
    if (p->hS) cudaFreeHost(p->hS);
    if (p->hIn) cudaFreeHost(p->hIn);
    if (p->hOut) cudaFreeHost(p->hOut);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
}

LaunchCtx ctx(vfem_problem* p) { return LaunchCtx{p->stream, p->S, p->rb, p->tma}; }

template <typename T>
vfem_status invertCoarse(vfem_problem* p, const float* E, double scale, T* K);

vfem_status buildCoarse(vfem_problem* p) {
    DevLevel& dc = p->L.back();
    // Coarsest free DOFs (FEM.cpp:473-496), in compressed (storage) order, from the level's flags.
    {
        std::vector<uint8_t> fl((size_t)dc.g.nnode);
        CK(cudaMemcpyAsync(fl.data(), dc.flags, fl.size(), cudaMemcpyDeviceToHost, p->stream));
        CK(cudaStreamSynchronize(p->stream));
        p->coarseFreeDof.clear();
        p->coarseFreeNode.assign(fl.size(), -1);
        int32_t nf = 0;
        for (size_t s = 0; s < fl.size(); ++s) {
            if (!(fl[s] & FLAG_USED) || (fl[s] & FLAG_FIXED)) continue;
            p->coarseFreeNode[s] = nf++;
            for (int c = 0; c < 3; ++c) p->coarseFreeDof.push_back((int32_t)(3 * s + c));
        }
    }
    int64_t n = (int64_t)p->coarseFreeDof.size();
    p->nc = n;
    if (n > kMaxCoarseFree)
        return fail(VFEM_ERR_COARSE_TOO_LARGE, "coarsest level has " + std::to_string(n) +
                                                   " free DOFs; add levels (limit " +
                                                   std::to_string(kMaxCoarseFree) + ")");
    if (n == 0) return VFEM_OK;
    CK(upload(&p->freeDof, p->coarseFreeDof));
    CK(upload(&p->dFreeNode, p->coarseFreeNode));
    CK(dalloc(&p->cb64, coarseBlocks(n) * CT));
    CK(dalloc(&p->cb32, coarseBlocks(n) * CT));
    CK(dalloc(&p->cpart, coarseTiles(n) * 2 * CT));
    return VFEM_OK;
}

// cuSOLVER's dense Cholesky factorisation and inverse by scalar type.
struct SolverFp64 {
    typedef double T;
    static cusolverStatus_t potrfBuf(cusolverDnHandle_t h, int n, T* A, int* lw) {
        return cusolverDnDpotrf_bufferSize(h, CUBLAS_FILL_MODE_LOWER, n, A, n, lw);
    }
    static cusolverStatus_t potriBuf(cusolverDnHandle_t h, int n, T* A, int* lw) {
        return cusolverDnDpotri_bufferSize(h, CUBLAS_FILL_MODE_LOWER, n, A, n, lw);
    }
    static cusolverStatus_t potrf(cusolverDnHandle_t h, int n, T* A, T* w, int lw, int* info) {
        return cusolverDnDpotrf(h, CUBLAS_FILL_MODE_LOWER, n, A, n, w, lw, info);
    }
    static cusolverStatus_t potri(cusolverDnHandle_t h, int n, T* A, T* w, int lw, int* info) {
        return cusolverDnDpotri(h, CUBLAS_FILL_MODE_LOWER, n, A, n, w, lw, info);
    }
};
struct SolverFp32 {
    typedef float T;
    static cusolverStatus_t potrfBuf(cusolverDnHandle_t h, int n, T* A, int* lw) {
        return cusolverDnSpotrf_bufferSize(h, CUBLAS_FILL_MODE_LOWER, n, A, n, lw);
    }
    static cusolverStatus_t potriBuf(cusolverDnHandle_t h, int n, T* A, int* lw) {
        return cusolverDnSpotri_bufferSize(h, CUBLAS_FILL_MODE_LOWER, n, A, n, lw);
    }
    static cusolverStatus_t potrf(cusolverDnHandle_t h, int n, T* A, T* w, int lw, int* info) {
        return cusolverDnSpotrf(h, CUBLAS_FILL_MODE_LOWER, n, A, n, w, lw, info);
    }
    static cusolverStatus_t potri(cusolverDnHandle_t h, int n, T* A, T* w, int lw, int* info) {
        return cusolverDnSpotri(h, CUBLAS_FILL_MODE_LOWER, n, A, n, w, lw, info);
    }
};
template <typename T>
struct SolverOf;
template <>
struct SolverOf<double> {
    typedef SolverFp64 type;
};
template <>
struct SolverOf<float> {
    typedef SolverFp32 type;
};

// K = inverse of Kc = scale * sum_e E_e Ke on the coarsest free DOFs (assembleK,
// FEM.cpp:19-63,498-513): assembled on the GPU in T, cuSOLVER Cholesky (potrf)
// and inverse (potri) in T, symmetrised.  The FP32 inverse is factorised in
// FP32 (tens of milliseconds instead of seconds for the FP64 one on GB300).
// Coarsest systems beyond the 32-bit solver API (n^2 >= 2^31 values): 64-bit
// Cholesky (cusolverDnXpotrf), triangular inverse of the factor
// (cusolverDnXtrtri) and Kinv = L^-T L^-1 as one rank-n update (cuBLAS syrk,
// 64-bit sizes) into `work`, then copied back to K (lower triangle in cuSOLVER's
// column-major order; the caller symmetrises).
template <typename T>
vfem_status invertCoarseLarge(vfem_problem* p, T* K, int64_t n, cusolverDnHandle_t h) {
    const cudaDataType dt = std::is_same<T, double>::value ? CUDA_R_64F : CUDA_R_32F;
    cusolverDnParams_t params = nullptr;
    cublasHandle_t hb = nullptr;
    void* dws = nullptr;
    int* info = nullptr;
    T* C = nullptr;
    vfem_status st = VFEM_OK;
    size_t wd1 = 0, wh1 = 0, wd2 = 0, wh2 = 0;
    if (cusolverDnCreateParams(&params) != CUSOLVER_STATUS_SUCCESS || cublasCreate(&hb) != CUBLAS_STATUS_SUCCESS)
        st = fail(VFEM_ERR_CUDA, "cusolver/cublas handle");
    if (st == VFEM_OK) cublasSetStream(hb, p->stream);
    if (st == VFEM_OK &&
        (cusolverDnXpotrf_bufferSize(h, params, CUBLAS_FILL_MODE_LOWER, n, dt, K, n, dt, &wd1, &wh1) !=
             CUSOLVER_STATUS_SUCCESS ||
         cusolverDnXtrtri_bufferSize(h, CUBLAS_FILL_MODE_LOWER, CUBLAS_DIAG_NON_UNIT, n, dt, K, n, &wd2, &wh2) !=
             CUSOLVER_STATUS_SUCCESS))
        st = fail(VFEM_ERR_CUDA, "cusolver 64-bit buffer size query failed");
    std::vector<char> hws(std::max<size_t>(1, std::max(wh1, wh2)));
    if (st == VFEM_OK) {
        // the syrk result is a second n x n matrix: fail early, with the size, when it cannot fit
        const size_t need = sizeof(T) * (size_t)(n * n) + std::max(wd1, wd2);
        size_t freeB = 0, totalB = 0;
        if (cudaMemGetInfo(&freeB, &totalB) == cudaSuccess && freeB < need)
            st = fail(VFEM_ERR_OUT_OF_MEMORY, "coarse inverse of " + std::to_string(n) + " free DOFs needs " +
                                                  std::to_string(need >> 20) + " MiB more device memory (" +
                                                  std::to_string(freeB >> 20) + " MiB free)");
    }
    if (st == VFEM_OK && (cudaMalloc(&dws, std::max<size_t>(16, std::max(wd1, wd2))) != cudaSuccess ||
                          cudaMalloc(&info, sizeof(int)) != cudaSuccess || dalloc(&C, n * n) != cudaSuccess))
        st = fail(VFEM_ERR_OUT_OF_MEMORY, "coarse inverse workspace");
    auto checkInfo = [&](const char* what) {
        int hinfo = 0;
        cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, p->stream);
        if (cudaStreamSynchronize(p->stream) != cudaSuccess) return fail(VFEM_ERR_CUDA, what);
        if (hinfo != 0)
            return fail(VFEM_ERR_SINGULAR, std::string(what) + " (info " + std::to_string(hinfo) + ")");
        return VFEM_OK;
    };
    if (st == VFEM_OK) {
        if (cusolverDnXpotrf(h, params, CUBLAS_FILL_MODE_LOWER, n, dt, K, n, dt, dws, wd1, hws.data(), wh1, info) !=
            CUSOLVER_STATUS_SUCCESS)
            st = fail(VFEM_ERR_CUDA, "cusolverDnXpotrf failed");
        else
            st = checkInfo("coarsest system is not positive definite");
    }
    if (st == VFEM_OK) {
        if (cusolverDnXtrtri(h, CUBLAS_FILL_MODE_LOWER, CUBLAS_DIAG_NON_UNIT, n, dt, K, n, dws, wd2, hws.data(), wh2,
                             info) != CUSOLVER_STATUS_SUCCESS)
            st = fail(VFEM_ERR_CUDA, "cusolverDnXtrtri failed");
        else
            st = checkInfo("coarsest factor inverse failed");
    }
    if (st == VFEM_OK) {
        // syrk reads the whole of L^-1: clear its (column-major) upper triangle first
        p->launches += launchZeroStrictRowMajorLower<T>(p->stream, K, n);
        const T one = T(1), zero = T(0);
        cublasStatus_t bs;
        if constexpr (std::is_same<T, double>::value)
            bs = cublasDsyrk_64(hb, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, n, n, &one, K, n, &zero, C, n);
        else
            bs = cublasSsyrk_64(hb, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, n, n, &one, K, n, &zero, C, n);
        if (bs != CUBLAS_STATUS_SUCCESS) st = fail(VFEM_ERR_CUDA, "cublas syrk failed");
        else if (cudaMemcpyAsync(K, C, sizeof(T) * (size_t)(n * n), cudaMemcpyDeviceToDevice, p->stream) !=
                 cudaSuccess)
            st = fail(VFEM_ERR_CUDA, "coarse inverse copy");
    }
    if (cudaStreamSynchronize(p->stream) != cudaSuccess && st == VFEM_OK) st = fail(VFEM_ERR_CUDA, "coarse inverse");
    cudaFree(dws);
    cudaFree(info);
    cudaFree(C);
    if (hb) cublasDestroy(hb);
    if (params) cusolverDnDestroyParams(params);
    return st;
}

template <typename T>
vfem_status invertCoarse(vfem_problem* p, const float* E, double scale, T* K) {
    typedef typename SolverOf<T>::type Sv;
    DevLevel& dc = p->L.back();
    const int64_t n = p->nc;
    CK(cudaMemsetAsync(K, 0, sizeof(T) * (size_t)(n * n), p->stream));
    p->launches += launchAssembleCoarse<T>(p->stream, dc.g, E, p->dFreeNode, p->ke.Ke, scale, K, n);
    CK(cudaGetLastError());
    if (n > g_coarse64Min) {
        cusolverDnHandle_t hl = nullptr;
        if (cusolverDnCreate(&hl) != CUSOLVER_STATUS_SUCCESS) return fail(VFEM_ERR_CUDA, "cusolverDnCreate failed");
        cusolverDnSetStream(hl, p->stream);
        vfem_status sl = invertCoarseLarge<T>(p, K, n, hl);
        cusolverDnDestroy(hl);
        if (sl != VFEM_OK) return sl;
        p->launches += launchSymmetrizeLowerToFull<T>(p->stream, K, n);
        if (cudaStreamSynchronize(p->stream) != cudaSuccess) return fail(VFEM_ERR_CUDA, "coarse inverse kernels");
        return VFEM_OK;
    }
    cusolverDnHandle_t h = nullptr;
    if (cusolverDnCreate(&h) != CUSOLVER_STATUS_SUCCESS) return fail(VFEM_ERR_CUDA, "cusolverDnCreate failed");
    cusolverDnSetStream(h, p->stream);
    int lw1 = 0, lw2 = 0;
    vfem_status st = VFEM_OK;
    T* work = nullptr;
    int* info = nullptr;
    int hinfo = 0;
    if (Sv::potrfBuf(h, (int)n, K, &lw1) != CUSOLVER_STATUS_SUCCESS ||
        Sv::potriBuf(h, (int)n, K, &lw2) != CUSOLVER_STATUS_SUCCESS)
        st = fail(VFEM_ERR_CUDA, "cusolver buffer size query failed");
    const int lw = std::max(1, std::max(lw1, lw2));
    if (st == VFEM_OK && (cudaMalloc(&work, sizeof(T) * (size_t)lw) != cudaSuccess ||
                          cudaMalloc(&info, sizeof(int)) != cudaSuccess))
        st = fail(VFEM_ERR_OUT_OF_MEMORY, "cusolver workspace");
    if (st == VFEM_OK) {
        if (Sv::potrf(h, (int)n, K, work, lw, info) != CUSOLVER_STATUS_SUCCESS)
            st = fail(VFEM_ERR_CUDA, "cusolver potrf failed");
        else {
            cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, p->stream);
            cudaStreamSynchronize(p->stream);
            if (hinfo != 0) st = fail(VFEM_ERR_SINGULAR, "coarsest system is not positive definite (potrf info " +
                                                            std::to_string(hinfo) + ")");
        }
    }
    if (st == VFEM_OK) {
        if (Sv::potri(h, (int)n, K, work, lw, info) != CUSOLVER_STATUS_SUCCESS)
            st = fail(VFEM_ERR_CUDA, "cusolver potri failed");
        else {
            cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, p->stream);
            cudaStreamSynchronize(p->stream);
            if (hinfo != 0) st = fail(VFEM_ERR_SINGULAR, "coarsest inverse failed (potri info " +
                                                            std::to_string(hinfo) + ")");
        }
    }
    if (st == VFEM_OK) {
        p->launches += launchSymmetrizeLowerToFull<T>(p->stream, K, n);
        if (cudaStreamSynchronize(p->stream) != cudaSuccess) st = fail(VFEM_ERR_CUDA, "coarse inverse kernels");
    }
    cudaFree(work);
    cudaFree(info);
    cusolverDnDestroy(h);
    return st;
}

template <typename T>
vfem_status ensureCoarse(vfem_problem* p, bool vcycle);

// FP64: the full matrix, applied by a one-FMA-per-value GEMV.
template <>
vfem_status ensureCoarse<double>(vfem_problem* p, bool vcycle) {
    if (p->nc == 0) return VFEM_OK;
    double*& K = vcycle ? p->KinvV64 : p->Kinv64;
    if (K) return VFEM_OK;
    double* out = nullptr;
    CK(dalloc(&out, p->nc * p->nc));
    const DevLevel& dc = p->L.back();
    const vfem_status st = invertCoarse<double>(p, vcycle ? dc.Ev : dc.E, dc.scale, out);
    if (st != VFEM_OK) {
        cudaFree(out);
        return st;
    }
    K = out;
    return VFEM_OK;
}

// Mixed precision: factorised and inverted in FP32, stored as packed FP16
// tiles scaled by a power of two (the rounding error of the FP16 values,
// 2^-11 relative, is of the order of the FP32 inverse's own error for the
// coarse systems' condition numbers).  An FP32 factorisation that fails (a
// system too ill-conditioned for FP32) falls back to the FP64 inverse.
template <>
vfem_status ensureCoarse<float>(vfem_problem* p, bool vcycle) {
    if (p->nc == 0) return VFEM_OK;
    __half*& K = vcycle ? p->KinvVH : p->KinvH;
    if (K) return VFEM_OK;
    const int64_t n = p->nc;
    __half* out = nullptr;
    float* full = nullptr;
    CK(dalloc(&out, coarseTiles(n) * CT * CT));
    if (dalloc(&full, n * n + 1) != cudaSuccess) {
        cudaFree(out);
        return fail(VFEM_ERR_OUT_OF_MEMORY, "coarse inverse workspace");
    }
    const DevLevel& dc = p->L.back();
    vfem_status st = invertCoarse<float>(p, vcycle ? dc.Ev : dc.E, dc.scale, full);
    if (st == VFEM_ERR_SINGULAR) {
        st = ensureCoarse<double>(p, vcycle);
        if (st == VFEM_OK) p->launches += launchConvert<double, float>(p->stream, n * n, vcycle ? p->KinvV64 : p->Kinv64, full);
    }
    float maxDiag = 0.0f;
    if (st == VFEM_OK) {
        p->launches += launchMaxDiag(p->stream, full, n, full + n * n);
        if (cudaMemcpyAsync(&maxDiag, full + n * n, sizeof(float), cudaMemcpyDeviceToHost, p->stream) != cudaSuccess ||
            cudaStreamSynchronize(p->stream) != cudaSuccess)
            st = fail(VFEM_ERR_CUDA, "coarse inverse diagonal");
        else if (!(maxDiag > 0.0f) || !std::isfinite(maxDiag))
            st = fail(VFEM_ERR_SINGULAR, "coarsest inverse has no positive diagonal");
    }
    float& scale = vcycle ? p->scaleVH : p->scaleH;
    if (st == VFEM_OK) {
        // scale = 2^(e - 14) with maxDiag <= 2^e: stored diagonal in (2^13, 2^14].
        int e = 0;
        std::frexp(maxDiag, &e);
        scale = std::ldexp(1.0f, e - 14);
        p->launches += launchPackSymHalf(p->stream, full, n, 1.0f / scale, out);
        if (cudaStreamSynchronize(p->stream) != cudaSuccess) st = fail(VFEM_ERR_CUDA, "coarse inverse packing");
    }
    cudaFree(full);
    if (st != VFEM_OK) {
        cudaFree(out);
        return st;
    }
    K = out;
    return VFEM_OK;
}

// The hierarchy on the device (setup_gpu.cu): per level the element moduli,
// node flags, compressed numbering and inverse diagonals.  Only the level plan,
// the Galerkin child tables, the fixed-id check and the counters touch the host.
vfem_status buildHierarchyDevice(vfem_problem* p, const std::vector<LevelPlan>& plan, const uint8_t* vox,
                                 const float* Ein, const int64_t* fixed, int64_t nfixed) {
    const int L = (int)plan.size();
    p->L.resize(L);
    cudaStream_t st = p->stream;
    Diag24 dg;
    for (int i = 0; i < 24; ++i) dg.v[i] = p->ke.diag[i];
    SetupCounters* dcnt = nullptr;
    std::vector<SetupCounters> hcnt(L);
    CK(dalloc(&dcnt, (int64_t)L));
    int* scratch = nullptr;
    uint8_t* dvox = nullptr;
    float* dEin = nullptr;
    double* dtab = nullptr;
    int64_t* dfixed = nullptr;
    unsigned* dmax = nullptr;
    int32_t* store = nullptr;  // a level's compressed numbering before it is trimmed
    vfem_status result = VFEM_OK;
    auto cleanup = [&]() {
        cudaFree(dcnt); cudaFree(scratch); cudaFree(dvox); cudaFree(dEin); cudaFree(dtab); cudaFree(dfixed);
        cudaFree(dmax); cudaFree(store);
    };
#define CKS(call)                                                                                        \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess) {                                                                         \
            cleanup();                                                                                   \
            return fail(e_ == cudaErrorMemoryAllocation ? VFEM_ERR_OUT_OF_MEMORY : VFEM_ERR_CUDA,         \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                             \
        }                                                                                                \
    } while (0)
    const Grid& g0 = plan[0].g;
    const int64_t nvox = (int64_t)g0.ex * g0.ey * g0.ez;
    CKS(dalloc(&scratch, compactScratchInts(g0.nnode)));
    CKS(dalloc(&dvox, nvox));
    CKS(cudaMemcpyAsync(dvox, vox, (size_t)nvox, cudaMemcpyHostToDevice, st));
    if (Ein) {
        CKS(dalloc(&dEin, nvox));
        CKS(cudaMemcpyAsync(dEin, Ein, sizeof(float) * (size_t)nvox, cudaMemcpyHostToDevice, st));
    }
    for (int i = 0; i < L; ++i) {
        DevLevel& d = p->L[i];
        d.g = plan[i].g;
        d.div = plan[i].div;
        d.scale = plan[i].scale;
        const int64_t nn = d.g.nnode, nv = d.nvec();
        CKS(dalloc(&d.E, nn));
        CKS(dalloc(&d.flags, nn));
        CKS(dalloc(&d.dinv64, nv)); CKS(dalloc(&d.dinv32, nv));
        CKS(dalloc(&d.dinvR64, nv)); CKS(dalloc(&d.dinvR32, nv)); CKS(dalloc(&d.dinvH, nv));
        SetupCounters* c = dcnt + i;
        if (i == 0) {
            d.Ev = d.E;
            CKS(gpuLevel0(st, d.g, dvox, dEin, d.E, d.flags, c));
        } else {
            const DevLevel& f = p->L[i - 1];
            CKS(dalloc(&d.Ev, nn));
            CKS(gpuCoarseLevel(st, f.g, d.g, d.div, f.E, f.Ev, f.flags, d.E, d.Ev, d.flags, c));
        }
        // compressed numbering: sized by the node count, trimmed below
        CKS(dalloc(&store, nn));
        CKS(gpuCompactUsed(st, d.g, d.flags, scratch, store, c));
        CKS(cudaMemcpyAsync(&hcnt[i], c, sizeof(SetupCounters), cudaMemcpyDeviceToHost, st));
        CKS(cudaStreamSynchronize(st));
        if (i == 0) {
            if (hcnt[0].err & 2u) result = fail(VFEM_ERR_INVALID_ARGUMENT, "voxel values must be 0 or 1");
            else if (hcnt[0].err & 1u)
                result = fail(VFEM_ERR_INVALID_ARGUMENT, "non-positive or non-finite modulus on a filled voxel");
            else if (hcnt[0].filled == 0) result = fail(VFEM_ERR_EMPTY, "no filled voxel");
            for (int64_t k = 0; result == VFEM_OK && k < nfixed; ++k)
                if (fixed[k] < 0 || fixed[k] >= hcnt[0].nused)
                    result = fail(VFEM_ERR_INVALID_ARGUMENT, "fixed node id out of range");
        }
        if (result != VFEM_OK) {
            cleanup();
            return result;
        }
        d.nused = hcnt[i].nused;
        d.nelem = (int64_t)hcnt[i].nelem;
        CKS(dalloc(&d.nodeStore, d.nused));
        CKS(cudaMemcpyAsync(d.nodeStore, store, sizeof(int32_t) * (size_t)d.nused, cudaMemcpyDeviceToDevice, st));
        CKS(cudaStreamSynchronize(st));
        cudaFree(store);
        store = nullptr;
        if (i == 0) {
            if (nfixed > 0) {
                CKS(dalloc(&dfixed, nfixed));
                CKS(cudaMemcpyAsync(dfixed, fixed, sizeof(int64_t) * (size_t)nfixed, cudaMemcpyHostToDevice, st));
                CKS(gpuSetFixed(st, nfixed, dfixed, d.nodeStore, d.flags));
            }
            CKS(gpuDiagRedisc(st, d.g, d.E, d.flags, d.scale, dg, d.dinv64, d.dinv32));
        } else {
            const DevLevel& f = p->L[i - 1];
            std::vector<double> tab;
            childDiagTable(p->ke.Ke, d.div, tab);
            cudaFree(dtab);
            dtab = nullptr;
            CKS(upload(&dtab, tab));
            CKS(gpuDiagCoarse(st, f.g, d.g, d.div, f.E, d.E, d.flags, d.scale, std::pow(2.0, i - 1), dtab, dg,
                              d.dinv64, d.dinv32));
        }
        CKS(gpuDiagRedisc(st, d.g, d.Ev, d.flags, d.scale, dg, d.dinvR64, d.dinvR32));
        {
            // FP16 copy of dinv32: the smoothing term of the mixed V-cycle reads 2
            // bytes per value instead of 4 (a relative rounding of 2^-11 on a
            // Jacobi step of the preconditioner).
            if (!dmax) CKS(dalloc(&dmax, 1));
            CKS(cudaMemsetAsync(dmax, 0, sizeof(unsigned), st));
            p->launches += launchMaxAbs(st, d.dinv32, nv, dmax);
            unsigned bits = 0;
            CKS(cudaMemcpyAsync(&bits, dmax, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
            CKS(cudaStreamSynchronize(st));
            float mx = 0.0f;
            std::memcpy(&mx, &bits, sizeof(float));
            int e = 0;
            if (mx > 0.0f && std::isfinite(mx)) std::frexp(mx, &e);
            d.dinvHScale = std::ldexp(1.0f, e - 14);
            p->launches += launchToHalf(st, d.dinv32, nv, 1.0f / d.dinvHScale, d.dinvH);
        }
        p->launches += 8;
    }
    CKS(cudaStreamSynchronize(st));
#undef CKS
    cleanup();
    return VFEM_OK;
}

vfem_status createImpl(const uint8_t* vox, int nx, int ny, int nz, const double* Ke, const float* E,
                       const int64_t* fixed, int64_t nfixed, int numLevels, int skip, vfem_problem** out) {
    if (!vox || !Ke || !out || (nfixed > 0 && !fixed))
        return fail(VFEM_ERR_INVALID_ARGUMENT, "null pointer argument");
    if (nfixed <= 0)
        return fail(VFEM_ERR_INVALID_ARGUMENT, "no fixed nodes: the stiffness would be singular (rigid-body modes)");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(VFEM_ERR_NO_DEVICE, "no CUDA device");
    g_coarse64Min = std::max<long long>(1, envInt("VFEM_COARSE_64BIT_MIN", kMaxCoarse32));
    g_allocCountdown = std::max<long long>(0, envInt("VFEM_FAULT_ALLOC_AT", 0));
    vfem_problem* p = new vfem_problem();
    if (cudaGetDevice(&p->device) != cudaSuccess) {
        delete p;
        return fail(VFEM_ERR_CUDA, "cudaGetDevice");
    }
    vfem_status st = prepareKe(Ke, p->ke);
    if (st != VFEM_OK) {
        delete p;
        return fail(st, "Ke has non-finite entries");
    }
    {
        // Reducing kernels keep one partial per block; the largest grids are the
        // matvec tiles (31 x 7 x 32 owned nodes) and the 32 x 8 x 8-node per-node kernels.
        const int64_t gx = nx + 1, gy = ny + 1, gz = nz + 1;
        const int64_t mv = ((gx + 30) / 31) * ((gy + 6) / 7) * ((gz + 31) / 32);
        const int64_t pn = ((gx + 31) / 32) * ((gy + 7) / 8) * ((gz + 7) / 8);
        if (mv > kMaxRedBlocks || pn > kMaxRedBlocks) {
            delete p;
            return fail(VFEM_ERR_INVALID_ARGUMENT, "grid too large for the reduction buffer (" +
                                                       std::to_string(std::max(mv, pn)) + " blocks > " +
                                                       std::to_string(kMaxRedBlocks) + ")");
        }
    }
    std::string err;
    std::vector<LevelPlan> plan;
    st = planLevels(nx, ny, nz, numLevels, skip, plan, err);
    if (st != VFEM_OK) {
        delete p;
        return fail(st, err);
    }
    for (int i = 0; i < 45; ++i) {
        p->op64[i] = p->ke.ks[i];
        p->op32[i] = (float)p->ke.ks[i];
    }
    for (int i = 0; i < 576; ++i) {
        p->op64[45 + i] = p->ke.Ke[i];
        p->op32[45 + i] = (float)p->ke.Ke[i];
    }
    auto bail = [&](vfem_status s) {
        freeProblem(p);
        return s;
    };
#define CKP(call)                                                                                         \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess)                                                                            \
            return bail(fail(e_ == cudaErrorMemoryAllocation ? VFEM_ERR_OUT_OF_MEMORY : VFEM_ERR_CUDA,     \
                             std::string(#call) + ": " + cudaGetErrorString(e_)));                        \
    } while (0)
    CKP(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
    CKP(setKernelAttributes());
    // VFEM_TENSOR_CORE_PRODUCT=1: the FP32 CG product on the tensor cores (slower
    // than the CUDA-core kernel on GB300; kept as a measured alternative)
    p->tcReady = envInt("VFEM_TENSOR_CORE_PRODUCT", 0) != 0 && tcPrepare(p->ke.Ke, p->tc) &&
                 tcBlocks(plan[0].g) <= kMaxRedBlocks && tcSetAttributes() == cudaSuccess;
    // VFEM_TMA_MASK (default 0): bit 0 the FP32 restrictions with TMA-staged rows, bit 1 the
    // mixed up-leg with bulk-staged ranges; both measured slower than the direct-load kernels
    p->tma = tmaSetAttributes() == cudaSuccess ? (int)envInt("VFEM_TMA_MASK", 0) & 3 : 0;
    // The mixed solve's direction update (p = z + beta p, x += alpha p) runs inside
    // the CUDA-core CG product's input stage; VFEM_FUSED_DIRECTION=0 keeps the
    // separate kUpdatePX pass (the general-Ke and tensor-core products always do).
    p->pxFused = envInt("VFEM_FUSED_DIRECTION", 1) != 0 && p->ke.structured && !p->tcReady;
    st = buildHierarchyDevice(p, plan, vox, E, fixed, nfixed);
    if (st != VFEM_OK) return bail(st);
    for (DevLevel& d : p->L) {
        int64_t nv = d.nvec();
        CKP(dalloc(&d.r64, nv)); CKP(dalloc(&d.z64, nv)); CKP(dalloc(&d.t64, nv));
        CKP(dalloc(&d.r32, nv)); CKP(dalloc(&d.z32, nv)); CKP(dalloc(&d.t32, nv));
    }
    int64_t nv0 = p->L[0].nvec();
    CKP(dalloc(&p->f64, nv0)); CKP(dalloc(&p->x64, nv0)); CKP(dalloc(&p->p64, nv0)); CKP(dalloc(&p->Ap64, nv0));
    CKP(dalloc(&p->p32, nv0)); CKP(dalloc(&p->Ap32, nv0)); CKP(dalloc(&p->x32, nv0)); CKP(dalloc(&p->r32b, nv0));
    if (p->pxFused) CKP(dalloc(&p->p32b, nv0));
    if (!tmaAvailable(p->r32b, nv0)) p->tma &= ~1;
    CKP(dalloc(&p->S, 1));
    CKP(dalloc(&p->rb.partials, (int64_t)kMaxRedTerms * kMaxRedBlocks));
    CKP(dalloc(&p->rb.ticket, 1));
    CKP(dalloc(&p->dComp, 3 * p->L[0].nused));
    CKP(dalloc(&p->dFlag, 1));
    CKP(cudaMallocHost((void**)&p->hS, sizeof(Scalars)));
    CKP(cudaMallocHost((void**)&p->hIn, sizeof(double) * 3 * (size_t)std::max<int64_t>(1, p->L[0].nused)));
    CKP(cudaMallocHost((void**)&p->hOut, sizeof(double) * 3 * (size_t)std::max<int64_t>(1, p->L[0].nused)));
    st = buildCoarse(p);
    if (st == VFEM_OK) st = ensureCoarse<float>(p, false);  // the mixed solver's, and a check that Kc is SPD
    if (st != VFEM_OK) return bail(st);
    CKP(cudaStreamSynchronize(p->stream));
    CKP(cudaGetLastError());
    g_launches += p->launches;
    *out = p;
    return VFEM_OK;
#undef CKP
}

// ------------------------------------------------------------------ solver pieces
// Every helper returns the number of kernels it enqueued.

template <typename T>
T* lvR(DevLevel& l);
template <>
double* lvR<double>(DevLevel& l) { return l.r64; }
template <>
float* lvR<float>(DevLevel& l) { return l.r32; }
template <typename T>
T* lvZ(DevLevel& l);
template <>
double* lvZ<double>(DevLevel& l) { return l.z64; }
template <>
float* lvZ<float>(DevLevel& l) { return l.z32; }
template <typename T>
T* lvT(DevLevel& l);
template <>
double* lvT<double>(DevLevel& l) { return l.t64; }
template <>
float* lvT<float>(DevLevel& l) { return l.t32; }
// The mixed V-cycle's smoothing reads the FP16 inverse diagonal.
template <typename T>
HalfDiag halfDiag(const DevLevel& l) {
    return std::is_same<T, float>::value ? HalfDiag{l.dinvH, l.dinvHScale} : HalfDiag();
}
template <typename T>
T* lvDinv(DevLevel& l, bool redisc);
template <>
double* lvDinv<double>(DevLevel& l, bool redisc) { return redisc ? l.dinvR64 : l.dinv64; }
template <>
float* lvDinv<float>(DevLevel& l, bool redisc) { return redisc ? l.dinvR32 : l.dinv32; }
template <typename T>
const void* opc(vfem_problem* p);
template <>
const void* opc<double>(vfem_problem* p) { return p->op64; }
template <>
const void* opc<float>(vfem_problem* p) { return p->op32; }
template <typename T>
CoarseInv<T> kinv(vfem_problem* p, bool vcycle);
template <>
CoarseInv<double> kinv<double>(vfem_problem* p, bool vcycle) { return {vcycle ? p->KinvV64 : p->Kinv64}; }
template <>
CoarseInv<float> kinv<float>(vfem_problem* p, bool vcycle) {
    return vcycle ? CoarseInv<float>{p->KinvVH, p->scaleVH} : CoarseInv<float>{p->KinvH, p->scaleH};
}
template <typename T>
T* cbuf(vfem_problem* p);
template <>
double* cbuf<double>(vfem_problem* p) { return p->cb64; }
template <>
float* cbuf<float>(vfem_problem* p) { return p->cb32; }

template <typename T>
MatvecArgs<T> mvArgs(vfem_problem* p, int lv, const T* x, T* y, int mode) {
    DevLevel& l = p->L[lv];
    MatvecArgs<T> a{};
    a.g = l.g;
    a.E = l.E;
    a.flags = l.flags;
    a.x = x;
    a.y = y;
    a.scale = l.scale;
    a.mode = mode;
    a.checkDone = 1;
    return a;
}

// FP32 CG products (y = K x, fixed rows 0, x.(Kx)) run on the tensor cores when
// the problem was created with them enabled; every other product runs on the
// CUDA-core kernels.
template <typename T>
int matvec(vfem_problem* p, const MatvecArgs<T>& a, bool allowTc = true) {
    if constexpr (std::is_same<T, float>::value) {
        if (allowTc && p->tcReady && tcEligible(a)) return launchMatvecTC(ctx(p), a, p->tc);
    }
    return launchMatvec<T>(ctx(p), a, p->ke.structured, opc<T>(p));
}

// FP64 vectors, double-float arithmetic (the mixed solve's true residual).
int matvecDF(vfem_problem* p, const MatvecArgs<double>& a) {
    return launchMatvecDF(ctx(p), a, p->ke.structured, p->op64);
}

// z = M^-1 r on level `lv` (r, z given); returns kernels; on level 0 the final
// pass produces r.z (and z.aux) with epilogue `epi`.  *outZ receives the buffer
// holding the result (it differs from z in the multiplicative cycle when the
// number of post-sweeps is odd).
template <typename T>
int vcycle(vfem_problem* p, const vfem_options& o, int lv, T* r, T* z, T** outZ, const T* aux, int epi,
           bool restricted = false) {
    const int L = (int)p->L.size();
    int n = 0;
    DevLevel& l = p->L[lv];
    LaunchCtx c = ctx(p);
    if (lv == L - 1) {
        // Coarsest: exact dense-inverse solve on the free DOFs; fixed and unused DOFs stay 0.
        n += launchCoarseSolve<T>(c, kinv<T>(p, o.mg_mode == VFEM_MG_VCYCLE), p->nc, p->freeDof, r,
                                  cbuf<T>(p), reinterpret_cast<T*>(p->cpart), z, 1);
        if (lv == 0 && epi != EPI_NONE) n += launchDots<T>(c, l.nvec(), r, z, aux ? z : nullptr, aux, epi, 1);
        *outZ = z;
        return n;
    }
    DevLevel& lc = p->L[lv + 1];
    if (o.mg_mode == VFEM_MG_REFERENCE) {
        // Additive cycle of the reference (MultigridPreconditioner.hpp:158-193).
        // restricted: the caller has already restricted r (fused residual update).
        if (!restricted) n += launchRestrict<T>(c, l.g, lc.g, lc.div, r, lvR<T>(lc), 1);
        T* zc = nullptr;
        n += vcycle<T>(p, o, lv + 1, lvR<T>(lc), lvZ<T>(lc), &zc, nullptr, EPI_NONE);
        n += launchProlongSmooth<T>(c, l.g, lc.g, lc.div, zc, r, lvDinv<T>(l, false), l.flags, z, 2.0, lv == 0 ? 1 : 0,
                                    lv == 0 ? aux : nullptr, lv == 0 ? epi : EPI_NONE, 1, halfDiag<T>(l));
        *outZ = z;
        return n;
    }
    // Multiplicative V-cycle with damped Jacobi on the rediscretised level operators.
    const T* dinv = lvDinv<T>(l, true);
    T* cur = z;
    T* other = lvT<T>(l);
    n += launchJacobiZero<T>(c, l.g, r, dinv, l.flags, cur, o.omega, 1);
    for (int s = 1; s < o.pre_sweeps; ++s) {
        MatvecArgs<T> a = mvArgs<T>(p, lv, cur, other, MV_SMOOTH);
        a.E = l.Ev;
        a.f = r;
        a.dinv = dinv;
        a.omega = o.omega;
        n += matvec<T>(p, a);
        std::swap(cur, other);
    }
    {
        MatvecArgs<T> a = mvArgs<T>(p, lv, cur, other, MV_RESID0);
        a.E = l.Ev;
        a.f = r;
        n += matvec<T>(p, a);
    }
    n += launchRestrict<T>(c, l.g, lc.g, lc.div, other, lvR<T>(lc), 1);
    T* zc = nullptr;
    n += vcycle<T>(p, o, lv + 1, lvR<T>(lc), lvZ<T>(lc), &zc, nullptr, EPI_NONE);
    n += launchProlongAdd<T>(c, l.g, lc.g, lc.div, zc, l.flags, cur, 1);
    for (int s = 0; s < o.post_sweeps; ++s) {
        MatvecArgs<T> a = mvArgs<T>(p, lv, cur, other, MV_SMOOTH);
        a.E = l.Ev;
        a.f = r;
        a.dinv = dinv;
        a.omega = o.omega;
        if (lv == 0 && s == o.post_sweeps - 1 && epi != EPI_NONE) {
            a.dot0 = DOT_F_OUT;
            a.dot1 = aux ? 1 : 0;
            a.aux = aux;
            a.epi = epi;
        }
        n += matvec<T>(p, a);
        std::swap(cur, other);
    }
    if (lv == 0 && o.post_sweeps == 0 && epi != EPI_NONE)
        n += launchDots<T>(c, l.nvec(), r, cur, aux ? cur : nullptr, aux, epi, 1);
    *outZ = cur;
    return n;
}

template <typename T>
const T* coarseV(vfem_problem* p, bool kv);
template <>
const double* coarseV<double>(vfem_problem* p, bool kv) { return kv ? p->KV64 : p->V64; }
template <>
const float* coarseV<float>(vfem_problem* p, bool kv) { return kv ? p->KV32 : p->V32; }

// Preconditioner application on level 0 (identity when mg_mode == NONE).  With a
// coarse space V set, the result is the deflated (A-DEF2) form
//   z = M^-1 r + V G^-1 (V^T r - (KV)^T M^-1 r),  G = V^T K V,
// which for residuals orthogonal to V (those of deflated CG) is the projection
// (I - V G^-1 V^T K) M^-1 r that keeps every search direction K-orthogonal to V;
// the dots of `epi` (r.z, z.aux) are then taken on that z.
template <typename T>
int precondition(vfem_problem* p, const vfem_options& o, T* r, T* z, T** outZ, const T* aux, int epi,
                 bool restricted = false) {
    DevLevel& l = p->L[0];
    const bool cs = p->coarseK > 0;
    int n = 0;
    if (o.mg_mode == VFEM_MG_NONE) {
        n = launchConvert<T, T>(p->stream, l.nvec(), r, z);
        *outZ = z;
    } else {
        n = vcycle<T>(p, o, 0, r, z, outZ, cs ? nullptr : aux, cs ? EPI_NONE : epi, restricted);
        if (!cs) return n;
    }
    if (cs)
        n += launchCoarseSpace<T>(ctx(p), l.nvec(), p->coarseK, coarseV<T>(p, false), coarseV<T>(p, true), p->coarseG,
                                  r, *outZ, 1);
    if (epi != EPI_NONE) n += launchDots<T>(ctx(p), l.nvec(), r, *outZ, aux ? *outZ : nullptr, aux, epi, 1);
    return n;
}

// The mixed solve fuses its residual update with the first restriction of the
// reference cycle (2x first coarsening); the residual then alternates between
// two buffers from iteration to iteration.
bool fusedUpdateRestrict(const vfem_problem* p, const vfem_options& o) {
    return o.precision == VFEM_PREC_MIXED && o.mg_mode == VFEM_MG_REFERENCE && p->L.size() >= 2 && p->L[1].div == 2;
}

// One PCG iteration (after initialisation).  FP64: Eigen's loop body.
// Mixed: FP32 vectors, FP64 x, conditional FP64 true-residual pass.
int iteration(vfem_problem* p, const vfem_options& o, double** zOut64, float** zOut32, int parity) {
    DevLevel& l0 = p->L[0];
    const int64_t n = l0.nvec();
    LaunchCtx c = ctx(p);
    int k = 0;
    if (o.precision == VFEM_PREC_FP64) {
        MatvecArgs<double> a = mvArgs<double>(p, 0, p->p64, p->Ap64, MV_AX);
        a.dot0 = DOT_X_OUT;
        a.epi = EPI_ALPHA;
        k += matvec<double>(p, a);
        k += launchUpdateXR<double, double>(c, n, p->x64, l0.r64, p->p64, p->Ap64);
        double* z = nullptr;
        k += precondition<double>(p, o, l0.r64, l0.z64, &z, o.flexible ? p->Ap64 : nullptr, EPI_BETA);
        k += launchUpdateP<double>(c, n, p->p64, z, 0);
        *zOut64 = z;
    } else {
        MatvecArgs<float> a = mvArgs<float>(p, 0, p->p32, p->Ap32, MV_AX);
        a.dot0 = DOT_X_OUT;
        a.epi = EPI_ALPHA;
        if (p->pxFused) {
            // p = z + beta p and the previous iteration's x += alpha p, in the product
            a.zin = *zOut32;
            a.pAlt = p->p32b;
            a.xacc = p->x32;
            k += launchMatvecPX(c, a, static_cast<const float*>(opc<float>(p)));
        } else {
            k += matvec<float>(p, a);
        }
        // x += alpha p is deferred to the next product (or launchUpdatePX) / the flush
        const bool fused = fusedUpdateRestrict(p, o);
        float* r = l0.r32;
        if (fused) {
            float* rIn = parity ? p->r32b : l0.r32;
            r = parity ? l0.r32 : p->r32b;
            k += launchUpdateRestrict(c, l0.g, p->L[1].g, rIn, p->Ap32, r, p->L[1].r32);
        } else {
            k += launchUpdateR(c, n, r, p->Ap32);
        }
        k += launchFlushX(c, n, p->x64, p->x32, p->p32, p->p32b, 1);
        // True residual f - K x64 in double-float; only its FP32 rounding (the new
        // recursive residual) and its norm are kept.
        MatvecArgs<double> t = mvArgs<double>(p, 0, p->x64, nullptr, MV_RESID);
        t.f = p->f64;
        t.y32 = r;
        t.dot0 = DOT_OUT_OUT;
        t.epi = EPI_TRUE;
        t.condTrue = 1;
        k += matvecDF(p, t);
        // a replaced residual is restricted again
        if (fused) k += launchRestrict<float>(c, l0.g, p->L[1].g, 2, r, p->L[1].r32, 2);
        float* z = nullptr;
        k += precondition<float>(p, o, r, l0.z32, &z, o.flexible ? p->Ap32 : nullptr, EPI_BETA, fused);
        if (!p->pxFused) k += launchUpdatePX(c, n, p->p32, z, p->x32);
        *zOut32 = z;
    }
    return k;
}

vfem_status checkOptions(const vfem_options& o) {
    if (!(o.rtol > 0) || o.mg_mode < 0 || o.mg_mode > 2 || o.precision < 0 || o.precision > 1 ||
        (o.mg_mode == VFEM_MG_VCYCLE && (!(o.omega > 0) || o.pre_sweeps < 1 || o.post_sweeps < 0)) ||
        o.check_every < 1 || o.check_every > 1024 || o.replace_every < 0 ||
        !(o.replace_delta >= 0.0 && o.replace_delta < 1.0) || o.fallback_fp64 < 0 || o.fallback_fp64 > 1 ||
        o.debug_break_at < 0)
        return fail(VFEM_ERR_INVALID_ARGUMENT, "invalid solver options");
    return VFEM_OK;
}

// One solve with validated options o; x64 holds the initial guess when haveX0.
vfem_status solvePhase(vfem_problem* p, const vfem_options& o, bool haveX0, vfem_stats* st) {
    vfem_status s = o.precision == VFEM_PREC_FP64 ? ensureCoarse<double>(p, o.mg_mode == VFEM_MG_VCYCLE)
                                      : ensureCoarse<float>(p, o.mg_mode == VFEM_MG_VCYCLE);
    if (s != VFEM_OK) return s;
    DevLevel& l0 = p->L[0];
    const int64_t n = l0.nvec();
    const long long maxIter = o.max_iter > 0 ? o.max_iter : 2 * 3 * l0.nused;
    const bool mixed = o.precision == VFEM_PREC_MIXED;
    LaunchCtx c = ctx(p);
    long long launches = 0;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, p->stream));
    launches += launchInitScalars(p->stream, p->S, o.rtol, maxIter, o.flexible, mixed ? 1 : 0,
                                  mixed ? o.replace_every : 0, o.replace_delta, o.debug_break_at);
    // ---- initial residual, norms, first direction
    double* z64 = nullptr;
    float* z32 = nullptr;
    if (haveX0) {
        MatvecArgs<double> a = mvArgs<double>(p, 0, p->x64, l0.r64, MV_RESID);
        a.f = p->f64;
        a.checkDone = 0;
        if (mixed) {
            a.y32 = l0.r32;
            launches += matvecDF(p, a);
        } else {
            launches += matvec<double>(p, a);
        }
    } else {
        launches += launchFill<double>(p->stream, n, p->x64, 0.0);
        launches += launchConvert<double, double>(p->stream, n, p->f64, l0.r64);
        if (mixed) launches += launchConvert<double, float>(p->stream, n, p->f64, l0.r32);
    }
    if (p->coarseK > 0) {
        // deflated CG starts from x + V G^-1 V^T r, whose residual is orthogonal to V
        launches += launchCoarseStart(c, n, p->coarseK, p->V64, p->KV64, p->coarseG, p->x64, l0.r64);
        if (mixed) launches += launchConvert<double, float>(p->stream, n, l0.r64, l0.r32);
    }
    if (mixed) launches += launchFill<float>(p->stream, n, p->x32, 0.f);
    launches += launchDots<double>(c, n, p->f64, p->f64, l0.r64, l0.r64, EPI_INIT, 0);
    if (mixed) {
        launches += precondition<float>(p, o, l0.r32, l0.z32, &z32, nullptr, EPI_RHO0);
        // (fused: the first product forms p = z, beta being 0 in fresh scalars)
        if (!p->pxFused) launches += launchUpdateP<float>(c, n, p->p32, z32, 1);
    } else {
        launches += precondition<double>(p, o, l0.r64, l0.z64, &z64, nullptr, EPI_RHO0);
        launches += launchUpdateP<double>(c, n, p->p64, z64, 1);
    }
    CK(cudaGetLastError());
    // ---- chunked iterations replayed from a cached graph
    const int chunk = o.check_every;
    // With the fused residual update the residual alternates between two buffers,
    // so a chunk of odd length has a second graph for the other starting buffer.
    const int flip = fusedUpdateRestrict(p, o) ? (chunk & 1) : 0;
    auto graphFor = [&](int parity, CachedGraph** out) -> vfem_status {
        GraphKey key{o.mg_mode, o.precision, o.flexible, o.pre_sweeps, o.post_sweeps, mixed ? o.replace_every : 0,
                     o.check_every, o.omega, parity};
        CachedGraph& cg = p->graphs[key];
        if (!cg.exec) {
            cudaGraph_t graph = nullptr;
            CK(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
            long long k = 0;
            for (int i = 0; i < chunk; ++i) k += iteration(p, o, &z64, &z32, (parity + i) & 1);
            cudaError_t ec = cudaStreamEndCapture(p->stream, &graph);
            if (ec != cudaSuccess) return fail(VFEM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ec));
            ec = cudaGraphInstantiate(&cg.exec, graph, 0);
            cudaGraphDestroy(graph);
            if (ec != cudaSuccess) {
                cg.exec = nullptr;
                return fail(VFEM_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ec));
            }
            cg.kernels = k;
        }
        *out = &cg;
        return VFEM_OK;
    };
    CachedGraph* cgs[2] = {nullptr, nullptr};
    if ((s = graphFor(0, &cgs[0])) != VFEM_OK) return s;
    if (flip && (s = graphFor(1, &cgs[1])) != VFEM_OK) return s;
    int parity = 0;  // the residual starts in L[0].r32
    long long chunks = 0;
    const long long maxChunks = maxIter / chunk + 2;
    for (;;) {
        CK(cudaMemcpyAsync(p->hS, p->S, sizeof(Scalars), cudaMemcpyDeviceToHost, p->stream));
        CK(cudaStreamSynchronize(p->stream));
        if (p->hS->done != RUNNING || chunks >= maxChunks) break;
        CK(cudaGraphLaunch(cgs[parity]->exec, p->stream));
        launches += cgs[parity]->kernels;
        parity ^= flip;
        ++chunks;
    }
    if (mixed) launches += launchFlushX(c, n, p->x64, p->x32, p->p32, p->p32b, 0);  // fold the remaining correction
    CK(cudaEventRecord(e1, p->stream));
    CK(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    Scalars hs = *p->hS;
    // ---- true residual at exit (outside the timed solve for FP64)
    double relTrue = NAN;
    if (mixed && hs.done == CONVERGED && hs.replacements > 0 && hs.rhsNorm2 > 0) {
        relTrue = std::sqrt(hs.rrTrue / hs.rhsNorm2);
    } else if ((o.compute_true_residual || (mixed && hs.done != CONVERGED)) && hs.rhsNorm2 > 0) {
        // (a failed mixed solve always reports it: the FP64 fallback starts from x when it is finite)
        MatvecArgs<double> a = mvArgs<double>(p, 0, p->x64, l0.t64, MV_RESID);
        a.f = p->f64;
        a.checkDone = 0;
        a.dot0 = DOT_OUT_OUT;
        a.epi = EPI_STORE;
        launches += matvec<double>(p, a);
        CK(cudaMemcpyAsync(p->hS, p->S, sizeof(Scalars), cudaMemcpyDeviceToHost, p->stream));
        CK(cudaStreamSynchronize(p->stream));
        relTrue = std::sqrt(p->hS->red0 / hs.rhsNorm2);
    } else if (hs.rhsNorm2 == 0) {
        relTrue = 0.0;
    }
    CK(cudaGetLastError());
    p->launches += launches;
    g_launches += launches;
    vfem_status result = VFEM_OK;
    if (hs.kernelTimeout) result = VFEM_ERR_TIMEOUT;
    else if (hs.done == BREAKDOWN) result = VFEM_ERR_BREAKDOWN;
    else if (hs.done == MAXITER || hs.done == RUNNING || hs.done == STAGNATED) result = VFEM_ERR_NOT_CONVERGED;
    if (st) {
        st->iterations = hs.iter;
        st->matvecs = hs.matvecs;
        st->residual_replacements = hs.replacements;
        st->rel_residual = relTrue;
        st->recursive_rel_residual = hs.rhsNorm2 > 0 ? std::sqrt(hs.rr / hs.rhsNorm2) : 0.0;
        st->solve_ms = ms;
        st->kernel_launches = launches;
        st->status = result;
    }
    if (result == VFEM_ERR_TIMEOUT) g_lastError = "a kernel's bounded wait ran out (tensor-core product)";
    if (result == VFEM_ERR_BREAKDOWN) g_lastError = "PCG breakdown (p^T A p <= 0 or non-finite scalar)";
    if (result == VFEM_ERR_NOT_CONVERGED)
        g_lastError = hs.done == STAGNATED ? "mixed-precision true residual stagnated" : "maximum iterations reached";
    return result;
}

// The solve with its FP64 fallback: a mixed-precision solve that breaks down or
// stops short of rtol hands its iterate to plain FP64 MG-PCG (the reference's
// method), which gets the iterations left of the budget.
vfem_status solveImpl(vfem_problem* p, const vfem_options* optIn, bool haveX0, vfem_stats* st) {
    vfem_options o;
    vfem_options_default(&o);
    if (optIn) o = *optIn;
    vfem_status s = checkOptions(o);
    if (s != VFEM_OK) return s;
    CK(cudaSetDevice(p->device));
    vfem_stats s1;
    std::memset(&s1, 0, sizeof(s1));
    s = solvePhase(p, o, haveX0, &s1);
    const long long budget = o.max_iter > 0 ? o.max_iter : 2 * 3 * p->L[0].nused;
    const bool retry = o.precision == VFEM_PREC_MIXED && o.fallback_fp64 &&
                       (s == VFEM_ERR_BREAKDOWN || s == VFEM_ERR_NOT_CONVERGED) && s1.iterations < budget;
    if (!retry) {
        if (st) *st = s1;
        return s;
    }
    vfem_options o2 = o;
    o2.precision = VFEM_PREC_FP64;
    o2.max_iter = budget - s1.iterations;
    o2.debug_break_at = 0;
    o2.compute_true_residual = 1;
    vfem_stats s2;
    std::memset(&s2, 0, sizeof(s2));
    // The FP64 solve continues from the mixed iterate only when that is better
    // than zero (true relative residual below 1); a diverged iterate would
    // leave the recursive residual far from the true one.
    const bool fromIterate = std::isfinite(s1.rel_residual) && s1.rel_residual < 1.0;
    s = solvePhase(p, o2, fromIterate, &s2);
    // The recursive residual of the continued solve decides convergence as in
    // Eigen; the fallback also requires the true residual near the tolerance.
    if (s == VFEM_OK && !(s2.rel_residual <= 10.0 * o.rtol))
        s = fail(VFEM_ERR_NOT_CONVERGED, "FP64 fallback: true residual above 10 x rtol");
    if (st) {
        *st = s2;
        st->iterations = s1.iterations + s2.iterations;
        st->matvecs = s1.matvecs + s2.matvecs;
        st->residual_replacements = s1.residual_replacements;
        st->solve_ms = s1.solve_ms + s2.solve_ms;
        st->kernel_launches = s1.kernel_launches + s2.kernel_launches;
        st->fallback = 1;
        st->fallback_iterations = s2.iterations;
        st->status = s;
    }
    return s;
}

// memcpy split over host threads for large host <-> pinned copies (one thread
// copies ~10 GB/s on the Grace host; the staging copies are 8 bytes per DOF).
void hostCopy(void* dst, const void* src, size_t bytes) {
    const size_t kSlice = (size_t)32 << 20;
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    static const size_t cap = (size_t)std::max<long long>(1, envInt("VFEM_HOST_COPY_THREADS", 8));
    const size_t nt = std::min<size_t>({cap, (size_t)hw, (bytes + kSlice - 1) / kSlice});
    if (nt <= 1) {
        std::memcpy(dst, src, bytes);
        return;
    }
    const size_t chunk = (bytes / nt + 63) & ~(size_t)63;
    std::vector<std::thread> th;
    for (size_t t = 1; t < nt; ++t) {
        const size_t off = t * chunk;
        if (off >= bytes) break;
        const size_t len = std::min(chunk, bytes - off);
        th.emplace_back([=] { std::memcpy((char*)dst + off, (const char*)src + off, len); });
    }
    std::memcpy(dst, src, std::min(chunk, bytes));
    for (auto& t : th) t.join();
}

// Host compressed vector -> dense device vector of level lv.  checkFinite: the
// scatter flags non-finite input (read back by the caller after a sync).
vfem_status toDenseHost(vfem_problem* p, int lv, const double* host, double* dense, bool checkFinite) {
    DevLevel& l = p->L[lv];
    hostCopy(p->hIn, host, sizeof(double) * 3 * (size_t)l.nused);
    CK(cudaMemcpyAsync(p->dComp, p->hIn, sizeof(double) * 3 * (size_t)l.nused, cudaMemcpyHostToDevice, p->stream));
    CK(cudaMemsetAsync(dense, 0, sizeof(double) * (size_t)l.nvec(), p->stream));
    if (checkFinite) CK(cudaMemsetAsync(p->dFlag, 0, sizeof(unsigned), p->stream));
    p->launches += launchScatterCompressed<double>(p->stream, l.nused, l.nodeStore, p->dComp, dense,
                                                   checkFinite ? p->dFlag : nullptr);
    g_launches += 1;
    return VFEM_OK;
}

vfem_status fromDenseHost(vfem_problem* p, int lv, const double* dense, double* host) {
    DevLevel& l = p->L[lv];
    p->launches += launchGatherCompressed<double>(p->stream, l.nused, l.nodeStore, dense, p->dComp);
    g_launches += 1;
    CK(cudaMemcpyAsync(p->hOut, p->dComp, sizeof(double) * 3 * (size_t)l.nused, cudaMemcpyDeviceToHost, p->stream));
    CK(cudaStreamSynchronize(p->stream));
    hostCopy(host, p->hOut, sizeof(double) * 3 * (size_t)l.nused);
    return VFEM_OK;
}

}  // namespace

// ------------------------------------------------------------------ C ABI
extern "C" {

void vfem_options_default(vfem_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->rtol = 1e-6;
    o->max_iter = 0;
    o->mg_mode = VFEM_MG_REFERENCE;
    o->precision = VFEM_PREC_FP64;
    o->omega = 0.6;
    o->pre_sweeps = 1;
    o->post_sweeps = 1;
    o->replace_every = 0;
    o->flexible = 0;
    o->check_every = 8;
    o->compute_true_residual = 1;
    o->replace_delta = 0.05;
    o->fallback_fp64 = 1;
    o->debug_break_at = 0;
}

const char* vfem_status_string(vfem_status s) {
    switch (s) {
        case VFEM_OK: return "ok";
        case VFEM_ERR_INVALID_ARGUMENT: return "invalid argument";
        case VFEM_ERR_CUDA: return "CUDA error";
        case VFEM_ERR_OUT_OF_MEMORY: return "out of device memory";
        case VFEM_ERR_NOT_CONVERGED: return "not converged";
        case VFEM_ERR_BREAKDOWN: return "PCG breakdown";
        case VFEM_ERR_SINGULAR: return "coarsest system singular";
        case VFEM_ERR_EMPTY: return "empty domain";
        case VFEM_ERR_COARSE_TOO_LARGE: return "coarsest level too large";
        case VFEM_ERR_NO_DEVICE: return "no CUDA device";
        case VFEM_ERR_TIMEOUT: return "timeout";
    }
    return "unknown status";
}

const char* vfem_last_error_message(void) { return g_lastError.c_str(); }

int64_t vfem_kernel_launch_count(void) { return g_launches.load(); }

vfem_status vfem_hex8_stiffness(double E, double nu, double* Ke) {
    if (!Ke || !(E > 0) || !(nu > -1.0 && nu < 0.5)) return fail(VFEM_ERR_INVALID_ARGUMENT, "bad E or nu");
    hex8Stiffness(E, nu, Ke);
    return VFEM_OK;
}

vfem_status vfem_problem_create(const uint8_t* voxels, int32_t nx, int32_t ny, int32_t nz, const double* Ke,
                                const float* E_or_null, const int64_t* fixed_nodes, int64_t nfixed,
                                int32_t num_levels, int32_t skip_levels, vfem_problem** out) {
    if (out) *out = nullptr;
    const vfem_status s =
        createImpl(voxels, nx, ny, nz, Ke, E_or_null, fixed_nodes, nfixed, num_levels, skip_levels, out);
    g_allocCountdown = 0;  // the allocation-failure hook covers one set-up only
    return s;
}

void vfem_problem_destroy(vfem_problem* p) { freeProblem(p); }

vfem_status vfem_problem_info(const vfem_problem* p, int32_t level, int64_t* num_nodes, int64_t* num_elements,
                              int32_t* num_levels, int64_t* coarse_free_dofs) {
    if (!p) return fail(VFEM_ERR_INVALID_ARGUMENT, "null problem");
    if (level < 0 || level >= (int)p->L.size()) return fail(VFEM_ERR_INVALID_ARGUMENT, "level out of range");
    if (num_nodes) *num_nodes = p->L[level].nused;
    if (num_elements) *num_elements = p->L[level].nelem;
    if (num_levels) *num_levels = (int32_t)p->L.size();
    if (coarse_free_dofs) *coarse_free_dofs = p->nc;
    return VFEM_OK;
}

vfem_status vfem_problem_set_rhs(vfem_problem* p, const double* f) {
    if (!p || !f) return fail(VFEM_ERR_INVALID_ARGUMENT, "null argument");
    CK(cudaSetDevice(p->device));
    p->rhsSet = false;
    vfem_status s = toDenseHost(p, 0, f, p->f64, true);
    if (s != VFEM_OK) return s;
    unsigned bad = 0;
    CK(cudaMemcpyAsync(&bad, p->dFlag, sizeof(unsigned), cudaMemcpyDeviceToHost, p->stream));
    CK(cudaStreamSynchronize(p->stream));
    if (bad) return fail(VFEM_ERR_INVALID_ARGUMENT, "non-finite right-hand side");
    p->rhsSet = true;
    return VFEM_OK;
}

vfem_status vfem_problem_set_loads(vfem_problem* p, const int64_t* nodes, const double* loads, int64_t n) {
    if (!p || (n > 0 && (!nodes || !loads)) || n < 0) return fail(VFEM_ERR_INVALID_ARGUMENT, "null argument");
    const int64_t nn = p->L[0].nused;
    std::vector<double> f(3 * (size_t)nn, 0.0);
    for (int64_t k = 0; k < n; ++k) {
        if (nodes[k] < 0 || nodes[k] >= nn) return fail(VFEM_ERR_INVALID_ARGUMENT, "load node id out of range");
        for (int c = 0; c < 3; ++c) f[3 * nodes[k] + c] = loads[3 * k + c];
    }
    return vfem_problem_set_rhs(p, f.data());
}

vfem_status vfem_solve_device(vfem_problem* p, const vfem_options* opt, double* u_out, vfem_stats* st) {
    if (!p) return fail(VFEM_ERR_INVALID_ARGUMENT, "null problem");
    if (!p->rhsSet) return fail(VFEM_ERR_INVALID_ARGUMENT, "right-hand side not set");
    if (st) std::memset(st, 0, sizeof(*st));
    vfem_status s = solveImpl(p, opt, false, st);
    if (u_out && (s == VFEM_OK || s == VFEM_ERR_NOT_CONVERGED)) {
        vfem_status s2 = fromDenseHost(p, 0, p->x64, u_out);
        if (s2 != VFEM_OK) return s2;
    }
    return s;
}

vfem_status vfem_solve(vfem_problem* p, const vfem_options* opt, const double* u0, double* u_out, vfem_stats* st) {
    if (!p || !u_out) return fail(VFEM_ERR_INVALID_ARGUMENT, "null argument");
    if (!p->rhsSet) return fail(VFEM_ERR_INVALID_ARGUMENT, "right-hand side not set");
    CK(cudaSetDevice(p->device));
    if (st) std::memset(st, 0, sizeof(*st));
    if (u0) {
        vfem_status s0 = toDenseHost(p, 0, u0, p->x64, false);
        if (s0 != VFEM_OK) return s0;
    }
    vfem_status s = solveImpl(p, opt, u0 != nullptr, st);
    if (s == VFEM_OK || s == VFEM_ERR_NOT_CONVERGED) {
        vfem_status s2 = fromDenseHost(p, 0, p->x64, u_out);
        if (s2 != VFEM_OK) return s2;
    }
    return s;
}

vfem_status vfem_apply_operator(vfem_problem* p, const double* x, double* y) {
    if (!p || !x || !y) return fail(VFEM_ERR_INVALID_ARGUMENT, "null argument");
    CK(cudaSetDevice(p->device));
    vfem_status s = toDenseHost(p, 0, x, p->p64, false);
    if (s != VFEM_OK) return s;
    MatvecArgs<double> a = mvArgs<double>(p, 0, p->p64, p->Ap64, MV_AX);
    a.checkDone = 0;
    p->launches += matvec<double>(p, a);
    g_launches += 1;
    CK(cudaGetLastError());
    return fromDenseHost(p, 0, p->Ap64, y);
}

vfem_status vfem_apply_operator_mixed(vfem_problem* p, const double* x, double* y, double* xKx) {
    if (!p || !x || !y) return fail(VFEM_ERR_INVALID_ARGUMENT, "null argument");
    CK(cudaSetDevice(p->device));
    DevLevel& l0 = p->L[0];
    const int64_t n = l0.nvec();
    vfem_status s = toDenseHost(p, 0, x, p->p64, false);
    if (s != VFEM_OK) return s;
    int k = launchConvert<double, float>(p->stream, n, p->p64, p->p32);
    k += launchInitScalars(p->stream, p->S, 1e-6, 1, 0, 1, 0, 0.0);
    MatvecArgs<float> a = mvArgs<float>(p, 0, p->p32, p->Ap32, MV_AX);
    a.checkDone = 0;
    a.dot0 = DOT_X_OUT;
    a.epi = EPI_STORE;
    k += matvec<float>(p, a);
    k += launchConvert<float, double>(p->stream, n, p->Ap32, p->Ap64);
    p->launches += k;
    g_launches += k;
    CK(cudaGetLastError());
    s = fromDenseHost(p, 0, p->Ap64, y);  // synchronises the stream
    if (s != VFEM_OK) return s;
    CK(cudaMemcpy(p->hS, p->S, sizeof(Scalars), cudaMemcpyDeviceToHost));
    if (p->hS->kernelTimeout) return fail(VFEM_ERR_TIMEOUT, "a kernel's bounded wait ran out (tensor-core product)");
    if (xKx) *xKx = p->hS->red0;
    return VFEM_OK;
}

vfem_status vfem_problem_set_coarse_space(vfem_problem* p, const double* V, int32_t k) {
    if (!p || k < 0 || k > 4 || (k > 0 && !V)) return fail(VFEM_ERR_INVALID_ARGUMENT, "bad argument");
    CK(cudaSetDevice(p->device));
    DevLevel& l0 = p->L[0];
    const int64_t n = l0.nvec(), nc = 3 * l0.nused;
    for (auto& kv : p->graphs)  // captured graphs hold the old correction
        if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    p->graphs.clear();
    p->coarseK = 0;
    if (k == 0) return VFEM_OK;
    if (p->coarseCap < k) {
        cudaFree(p->V64); cudaFree(p->V32); cudaFree(p->KV64); cudaFree(p->KV32);
        p->V64 = p->KV64 = nullptr;
        p->V32 = p->KV32 = nullptr;
        p->coarseCap = 0;
        CK(dalloc(&p->V64, k * n));
        CK(dalloc(&p->V32, k * n));
        CK(dalloc(&p->KV64, k * n));
        CK(dalloc(&p->KV32, k * n));
        p->coarseCap = k;
    }
    // columns with their fixed DOFs zeroed (the space the solver's iterates live in)
    int64_t nfix = 0;
    vfem_status s = vfem_fixed_nodes(p, 0, nullptr, 0, &nfix);
    if (s != VFEM_OK) return s;
    std::vector<int64_t> fixedNodes((size_t)nfix);
    if (nfix > 0 && (s = vfem_fixed_nodes(p, 0, fixedNodes.data(), nfix, &nfix)) != VFEM_OK) return s;
    std::vector<double> Vm(V, V + (size_t)nc * k);
    for (int j = 0; j < k; ++j)
        for (int64_t id : fixedNodes)
            for (int c3 = 0; c3 < 3; ++c3) Vm[(size_t)j * nc + 3 * id + c3] = 0.0;
    // K V from the FP64 operator (fixed rows zeroed), then G = V^T K V on the host
    std::vector<double> KV((size_t)nc * k);
    for (int j = 0; j < k; ++j) {
        double* vj = p->V64 + (size_t)j * n;
        double* kvj = p->KV64 + (size_t)j * n;
        s = toDenseHost(p, 0, Vm.data() + (size_t)j * nc, vj, true);
        if (s != VFEM_OK) return s;
        MatvecArgs<double> a = mvArgs<double>(p, 0, vj, kvj, MV_AX);
        a.checkDone = 0;
        p->launches += matvec<double>(p, a);
        s = fromDenseHost(p, 0, kvj, KV.data() + (size_t)j * nc);
        if (s != VFEM_OK) return s;
        unsigned bad = 0;
        CK(cudaMemcpyAsync(&bad, p->dFlag, sizeof(unsigned), cudaMemcpyDeviceToHost, p->stream));
        CK(cudaStreamSynchronize(p->stream));
        if (bad) return fail(VFEM_ERR_INVALID_ARGUMENT, "coarse space: non-finite entry");
    }
    p->launches += launchConvert<double, float>(p->stream, k * n, p->V64, p->V32);
    p->launches += launchConvert<double, float>(p->stream, k * n, p->KV64, p->KV32);
    CK(cudaStreamSynchronize(p->stream));
    double G[16] = {0}, Gi[16] = {0};
    for (int a = 0; a < k; ++a)
        for (int b = 0; b < k; ++b) {
            double sum = 0.0;
            for (int64_t i = 0; i < nc; ++i) sum += Vm[(size_t)a * nc + i] * KV[(size_t)b * nc + i];
            G[4 * a + b] = sum;
        }
    // symmetrise, then invert by Gauss-Jordan with partial pivoting (k <= 4)
    double M[4][8] = {};
    for (int a = 0; a < k; ++a)
        for (int b = 0; b < k; ++b) {
            M[a][b] = 0.5 * (G[4 * a + b] + G[4 * b + a]);
            M[a][4 + b] = a == b ? 1.0 : 0.0;
        }
    for (int c = 0; c < k; ++c) {
        int piv = c;
        for (int r2 = c + 1; r2 < k; ++r2)
            if (std::fabs(M[r2][c]) > std::fabs(M[piv][c])) piv = r2;
        if (!(M[piv][c] > 0.0 || M[piv][c] < 0.0) || !std::isfinite(M[piv][c]))
            return fail(VFEM_ERR_INVALID_ARGUMENT, "coarse space: V^T K V is singular (dependent or fixed-only columns)");
        for (int q = 0; q < 8; ++q) std::swap(M[c][q], M[piv][q]);
        const double d = M[c][c];
        for (int q = 0; q < 8; ++q) M[c][q] /= d;
        for (int r2 = 0; r2 < k; ++r2)
            if (r2 != c) {
                const double f = M[r2][c];
                for (int q = 0; q < 8; ++q) M[r2][q] -= f * M[c][q];
            }
    }
    for (int a = 0; a < k; ++a)
        for (int b = 0; b < k; ++b) Gi[4 * a + b] = M[a][4 + b];
    std::memcpy(p->coarseG.Ginv, Gi, sizeof(Gi));
    p->coarseK = k;
    return VFEM_OK;
}

int32_t vfem_problem_uses_tensor_cores(const vfem_problem* p) { return p && p->tcReady ? 1 : 0; }

int32_t vfem_problem_uses_tma(const vfem_problem* p) { return p ? p->tma : 0; }

vfem_status vfem_apply_operator_device_noalloc(vfem_problem* p, const double* x_device, double* y_device,
                                               double* xKx_device, void* stream) {
    if (!p || !x_device || !y_device || !xKx_device) return fail(VFEM_ERR_INVALID_ARGUMENT, "null argument");
    CK(cudaSetDevice(p->device));  // the scratch set-up below runs with the problem's device current
    MatvecArgs<double> a = mvArgs<double>(p, 0, x_device, y_device, MV_AX);
    bool tooLarge = false;
    CK(launchMatvecNoAlloc(static_cast<cudaStream_t>(stream), a, p->ke.structured, p->op64, xKx_device, &tooLarge));
    if (tooLarge)
        return fail(VFEM_ERR_INVALID_ARGUMENT,
                    "grid too large for the no-allocation scratch (at most 65536 product blocks of 31x7x32 "
                    "nodes, about 760^3 nodes for a cube)");
    p->launches += 1;
    g_launches += 1;
    return VFEM_OK;
}

vfem_status vfem_apply_preconditioner(vfem_problem* p, int32_t mg_mode, const double* r, double* z) {
    if (!p || !r || !z || (mg_mode != VFEM_MG_REFERENCE && mg_mode != VFEM_MG_VCYCLE))
        return fail(VFEM_ERR_INVALID_ARGUMENT, "bad argument");
    CK(cudaSetDevice(p->device));
    DevLevel& l0 = p->L[0];
    vfem_status s = ensureCoarse<double>(p, mg_mode == VFEM_MG_VCYCLE);
    if (s != VFEM_OK) return s;
    s = toDenseHost(p, 0, r, l0.r64, false);
    if (s != VFEM_OK) return s;
    vfem_options o;
    vfem_options_default(&o);
    o.mg_mode = mg_mode;
    launchInitScalars(p->stream, p->S, 1e-6, 1, 0, 0, 0, 0.0);
    double* zo = nullptr;
    int k = 1 + precondition<double>(p, o, l0.r64, l0.z64, &zo, nullptr, EPI_NONE);
    p->launches += k;
    g_launches += k;
    CK(cudaGetLastError());
    return fromDenseHost(p, 0, zo, z);
}

vfem_status vfem_apply_preconditioner_mixed(vfem_problem* p, int32_t mg_mode, const double* r, double* z) {
    if (!p || !r || !z || (mg_mode != VFEM_MG_REFERENCE && mg_mode != VFEM_MG_VCYCLE))
        return fail(VFEM_ERR_INVALID_ARGUMENT, "bad argument");
    CK(cudaSetDevice(p->device));
    DevLevel& l0 = p->L[0];
    vfem_status s = ensureCoarse<float>(p, mg_mode == VFEM_MG_VCYCLE);
    if (s != VFEM_OK) return s;
    s = toDenseHost(p, 0, r, l0.r64, false);
    if (s != VFEM_OK) return s;
    vfem_options o;
    vfem_options_default(&o);
    o.mg_mode = mg_mode;
    o.precision = VFEM_PREC_MIXED;
    const int64_t n = l0.nvec();
    int k = launchConvert<double, float>(p->stream, n, l0.r64, l0.r32);
    k += launchInitScalars(p->stream, p->S, 1e-6, 1, 0, 1, 0, 0.0);
    float* zo = nullptr;
    k += precondition<float>(p, o, l0.r32, l0.z32, &zo, nullptr, EPI_NONE);
    k += launchConvert<float, double>(p->stream, n, zo, l0.z64);
    p->launches += k;
    g_launches += k;
    CK(cudaGetLastError());
    return fromDenseHost(p, 0, l0.z64, z);
}

vfem_status vfem_restrict(vfem_problem* p, int32_t level, const double* fine, double* coarse) {
    if (!p || !fine || !coarse || level < 0 || level + 1 >= (int)p->L.size())
        return fail(VFEM_ERR_INVALID_ARGUMENT, "bad argument");
    CK(cudaSetDevice(p->device));
    DevLevel& lf = p->L[level];
    DevLevel& lc = p->L[level + 1];
    vfem_status s = toDenseHost(p, level, fine, lf.t64, false);
    if (s != VFEM_OK) return s;
    launchInitScalars(p->stream, p->S, 1e-6, 1, 0, 0, 0, 0.0);
    int k = 1 + launchRestrict<double>(ctx(p), lf.g, lc.g, lc.div, lf.t64, lc.t64, 0);
    p->launches += k;
    g_launches += k;
    CK(cudaGetLastError());
    return fromDenseHost(p, level + 1, lc.t64, coarse);
}

vfem_status vfem_interpolate(vfem_problem* p, int32_t level, const double* coarse, double* fine) {
    if (!p || !fine || !coarse || level < 0 || level + 1 >= (int)p->L.size())
        return fail(VFEM_ERR_INVALID_ARGUMENT, "bad argument");
    CK(cudaSetDevice(p->device));
    DevLevel& lf = p->L[level];
    DevLevel& lc = p->L[level + 1];
    vfem_status s = toDenseHost(p, level + 1, coarse, lc.t64, false);
    if (s != VFEM_OK) return s;
    launchInitScalars(p->stream, p->S, 1e-6, 1, 0, 0, 0, 0.0);
    CK(cudaMemsetAsync(lf.t64, 0, sizeof(double) * (size_t)lf.nvec(), p->stream));
    // Masked trilinear prolongation only: coefficient 0 on the Jacobi term, no fixed mask
    // (the reference's interpolate does not zero fixed nodes).
    int k = 1 + launchProlongSmooth<double>(ctx(p), lf.g, lc.g, lc.div, lc.t64, lf.t64, lf.dinv64, lf.flags, lf.z64,
                                            0.0, 0, nullptr, EPI_NONE, 0);
    p->launches += k;
    g_launches += k;
    CK(cudaGetLastError());
    return fromDenseHost(p, level, lf.z64, fine);
}

vfem_status vfem_profile_kernels(vfem_problem* p, int32_t reps, double* ms) {
    if (!p || !ms || reps < 1) return fail(VFEM_ERR_INVALID_ARGUMENT, "bad argument");
    CK(cudaSetDevice(p->device));
    vfem_status sc = ensureCoarse<double>(p, false);
    if (sc == VFEM_OK) sc = ensureCoarse<float>(p, false);
    if (sc != VFEM_OK) return sc;
    DevLevel& l0 = p->L[0];
    const bool two = p->L.size() > 1;
    DevLevel& l1 = p->L[two ? 1 : 0];
    const int64_t n = l0.nvec();
    LaunchCtx c = ctx(p);
    // Scalars with alpha = beta = 0 and done = 0: every kernel runs in full, vectors stay put.
    launchInitScalars(p->stream, p->S, 1e-6, 1 << 30, 0, 0, 0, 0.0);
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    long long launched = 1;
    bool pxScalars = false;
    for (int k = 0; k < VFEM_K_COUNT; ++k) {
        auto one = [&]() -> int {
            switch (k) {
                case VFEM_K_MATVEC_FP32_PX: {
                    if (!p->pxFused) return 0;
                    if (!pxScalars) {  // nonzero alpha and beta: the update runs in full (first, untimed call)
                        static const double half = 0.5;
                        char* sb = reinterpret_cast<char*>(p->S);
                        if (cudaMemcpyAsync(sb + offsetof(Scalars, alpha), &half, sizeof(double),
                                            cudaMemcpyHostToDevice, p->stream) != cudaSuccess ||
                            cudaMemcpyAsync(sb + offsetof(Scalars, beta), &half, sizeof(double),
                                            cudaMemcpyHostToDevice, p->stream) != cudaSuccess)
                            return 0;
                        pxScalars = true;
                    }
                    MatvecArgs<float> a = mvArgs<float>(p, 0, p->p32, p->Ap32, MV_AX);
                    a.dot0 = DOT_X_OUT;
                    a.epi = EPI_STORE;
                    a.zin = l0.z32;
                    a.pAlt = p->p32b;
                    a.xacc = p->x32;
                    return launchMatvecPX(c, a, static_cast<const float*>(opc<float>(p)));
                }
                case VFEM_K_MATVEC_FP64: {
                    MatvecArgs<double> a = mvArgs<double>(p, 0, p->p64, p->Ap64, MV_AX);
                    a.dot0 = DOT_X_OUT;
                    a.epi = EPI_STORE;
                    return matvec<double>(p, a);
                }
                case VFEM_K_MATVEC_FP32:
                case VFEM_K_MATVEC_FP32_SIMT: {
                    MatvecArgs<float> a = mvArgs<float>(p, 0, p->p32, p->Ap32, MV_AX);
                    a.dot0 = DOT_X_OUT;
                    a.epi = EPI_STORE;
                    return matvec<float>(p, a, k == VFEM_K_MATVEC_FP32);
                }
                case VFEM_K_RESTRICT_FP64:
                    return two ? launchRestrict<double>(c, l0.g, l1.g, l1.div, l0.r64, l1.r64, 1) : 0;
                case VFEM_K_RESTRICT_FP32:
                    return two ? launchRestrict<float>(c, l0.g, l1.g, l1.div, l0.r32, l1.r32, 1) : 0;
                case VFEM_K_UPDATE_RESTRICT_MIXED:
                    return two && l1.div == 2 ? launchUpdateRestrict(c, l0.g, l1.g, l0.r32, p->Ap32, p->r32b, l1.r32)
                                              : 0;
                case VFEM_K_PROLONG_FP64:
                    return two ? launchProlongSmooth<double>(c, l0.g, l1.g, l1.div, l1.z64, l0.r64, l0.dinv64, l0.flags,
                                                             l0.z64, 2.0, 1, nullptr, EPI_STORE, 1)
                               : 0;
                case VFEM_K_PROLONG_FP32:
                    return two ? launchProlongSmooth<float>(c, l0.g, l1.g, l1.div, l1.z32, l0.r32, l0.dinv32, l0.flags,
                                                            l0.z32, 2.0, 1, nullptr, EPI_STORE, 1, halfDiag<float>(l0))
                               : 0;
                case VFEM_K_UPDATE_XR_FP64:
                    return launchUpdateXR<double, double>(c, n, p->x64, l0.r64, p->p64, p->Ap64);
                case VFEM_K_UPDATE_XR_MIXED:
                    return launchUpdateR(c, n, l0.r32, p->Ap32);
                case VFEM_K_UPDATE_P_FP64:
                    return launchUpdateP<double>(c, n, p->p64, l0.z64, 0);
                case VFEM_K_UPDATE_P_FP32:
                    return launchUpdatePX(c, n, p->p32, l0.z32, p->x32);
                case VFEM_K_COARSE_FP64: {
                    DevLevel& lc = p->L.back();
                    return launchCoarseSolve<double>(c, kinv<double>(p, false), p->nc, p->freeDof, lc.r64, p->cb64, p->cpart,
                                                     lc.z64, 1);
                }
                case VFEM_K_COARSE_FP32: {
                    DevLevel& lc = p->L.back();
                    return launchCoarseSolve<float>(c, kinv<float>(p, false), p->nc, p->freeDof, lc.r32, p->cb32,
                                                    reinterpret_cast<float*>(p->cpart), lc.z32, 1);
                }
                default: {
                    MatvecArgs<double> a = mvArgs<double>(p, 0, p->x64, nullptr, MV_RESID);
                    a.f = p->f64;
                    a.y32 = l0.t32;
                    a.dot0 = DOT_OUT_OUT;
                    a.epi = EPI_STORE;
                    return matvecDF(p, a);
                }
            }
        };
        launched += one() + one();
        CK(cudaEventRecord(e0, p->stream));
        int cnt = 0;
        for (int r = 0; r < reps; ++r) cnt += one();
        CK(cudaEventRecord(e1, p->stream));
        CK(cudaEventSynchronize(e1));
        launched += cnt;
        float t = 0;
        cudaEventElapsedTime(&t, e0, e1);
        ms[k] = cnt ? (double)t / reps : 0.0;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    p->launches += launched;
    g_launches += launched;
    CK(cudaGetLastError());
    return VFEM_OK;
}

vfem_status vfem_inverse_diagonal(vfem_problem* p, int32_t level, double* out) {
    if (!p || !out || level < 0 || level >= (int)p->L.size()) return fail(VFEM_ERR_INVALID_ARGUMENT, "bad argument");
    CK(cudaSetDevice(p->device));
    return fromDenseHost(p, level, p->L[level].dinv64, out);
}

vfem_status vfem_fixed_nodes(vfem_problem* p, int32_t level, int64_t* out, int64_t cap, int64_t* count) {
    if (!p || level < 0 || level >= (int)p->L.size()) return fail(VFEM_ERR_INVALID_ARGUMENT, "bad argument");
    CK(cudaSetDevice(p->device));
    const DevLevel& l = p->L[level];
    std::vector<uint8_t> fl((size_t)l.g.nnode);
    std::vector<int32_t> store((size_t)l.nused);
    CK(cudaMemcpyAsync(fl.data(), l.flags, fl.size(), cudaMemcpyDeviceToHost, p->stream));
    CK(cudaMemcpyAsync(store.data(), l.nodeStore, sizeof(int32_t) * store.size(), cudaMemcpyDeviceToHost, p->stream));
    CK(cudaStreamSynchronize(p->stream));
    int64_t n = 0;
    for (size_t i = 0; i < store.size(); ++i) {
        if (!(fl[store[i]] & FLAG_FIXED)) continue;
        if (out && n < cap) out[n] = (int64_t)i;
        ++n;
    }
    if (count) *count = n;
    return VFEM_OK;
}

}  // extern "C"
