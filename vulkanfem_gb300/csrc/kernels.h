// kernels.h -- launch interface of the sm_103a kernels (kernels.cu).
//
// All kernels run on one stream in a fixed order, so they share one
// reduction buffer (block partials + ticket).  Solver scalars live in device
// memory (Scalars) so that a whole PCG iteration runs without a host round
// trip: each kernel returns immediately once `done` is set, and the host polls
// `done` once per chunk of iterations.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "vfem_internal.h"

namespace vfem {

// STAGNATED (mixed precision): three replacements in a row found the true
// residual no more than 1% below the previous one.
enum Done : int { RUNNING = 0, CONVERGED = 1, MAXITER = 2, BREAKDOWN = 3, STAGNATED = 4 };

struct Scalars {
    double rhsNorm2, threshold, tol2;
    double rho, rhoOld, pAp, rr, alpha, beta, zAp, rrTrue;
    double red0, red1;
    double rrLast;     // r.r at the last true-residual replacement (mixed precision)
    double delta2;     // replace when r.r < delta2 * rrLast (reliable-update criterion)
    long long iter, maxIter, matvecs, replacements;
    int done;
    int checkPending;  // mixed precision: recursive residual passed, verify in FP64
    int flexible;
    int mixed;
    int replaceEvery;
    int breakAt;       // testing: pAp of this iteration (1-based) is taken as -1 (0 = off)
    // mixed precision, deferred x += alpha p: value of `matvecs` when the
    // residual update last ran, when a conditional kFlushX folded alpha p, when
    // kUpdatePX ran; replStamp: when the true residual last replaced r
    long long rStamp, foldStamp, pxStamp, replStamp;
    double rrTruePrev;  // true r.r of the previous replacement
    long long stalls;   // consecutive replacements without a 1% drop of the true residual
    int kernelTimeout;  // a kernel's bounded wait ran out (the solve stops with BREAKDOWN)
    int pSel;           // fused direction update: 0 = the current p is in the first buffer, 1 = in the second
    double coarseCoef[4];  // coarse-space coefficients G^-1 (V^T r - (KV)^T z) of the current application
};

// Deflation coarse space of k <= 4 columns V (dense storage, column j at V + j * n),
// their products KV stored the same way, and G^-1 = (V^T K V)^-1 row-major 4 x 4.
struct CoarseSpace {
    double Ginv[16];
};

struct RedBuf {
    double* partials;   // kMaxRedTerms * kMaxRedBlocks (term k of block b at k * kMaxRedBlocks + b)
    unsigned* ticket;
};

constexpr int kMaxRedBlocks = 1 << 16;
// Sums one grid reduction carries at most (the partials buffer holds
// kMaxRedTerms * kMaxRedBlocks doubles; the deflation dots use 4).
constexpr int kMaxRedTerms = 4;

// What the last block of a reducing kernel does with the totals (t0, t1).
enum Epi : int {
    EPI_NONE = 0,
    EPI_STORE = 1,   // red0 = t0, red1 = t1
    EPI_ALPHA = 2,   // pAp = t0 -> alpha = rho / pAp
    EPI_CONV = 3,    // rr = t0 -> convergence test
    EPI_RHO0 = 4,    // rho = t0 (r.z of the first preconditioned residual)
    EPI_BETA = 5,    // rho = t0, zAp = t1 -> beta, iteration count
    EPI_INIT = 6,    // rhsNorm2 = t0, rr = t1 -> threshold
    EPI_TRUE = 7     // rrTrue = t0 (FP64 residual) -> replacement / final check
};

// Matvec output modes.
enum MvMode : int {
    MV_AX = 0,       // y = A x (fixed rows zeroed)
    MV_RESID = 1,    // y = f - A x
    MV_RESID0 = 2,   // y = f - A x, zero at fixed nodes
    MV_SMOOTH = 3    // y = x + omega D^-1 (f - A x), zero at fixed nodes
};

// Dot selections of a matvec / prolongation pass.
enum DotSel : int { DOT_NONE = 0, DOT_X_OUT = 1, DOT_OUT_OUT = 2, DOT_F_OUT = 3 };

template <typename T>
struct MatvecArgs {
    Grid g;
    const float* E;
    const uint8_t* flags;
    const T* x;
    T* y;
    const T* f;        // MV_RESID*, MV_SMOOTH
    const T* dinv;     // MV_SMOOTH
    const T* aux;      // second dot: out . aux
    float* y32;        // optional FP32 copy of y (mixed-precision residual replacement)
    double scale;      // operator multiplier on this level
    double omega;
    int mode, dot0, dot1, epi;
    int condTrue;      // run only when a true-residual pass is due (mixed precision)
    int checkDone;
    // Direction update fused into the FP32 CG product (launchMatvecPX): the
    // product's input is p = z + beta p_old, with p_old in x or pAlt and the new
    // p written to the other one (Scalars::pSel says which holds the current p),
    // and the deferred x += alpha p_old goes into xacc.
    const T* zin;
    T* pAlt;
    float* xacc;
};

struct OpConst64 { double ks[45]; double ke[576]; };
struct OpConst32 { float ks[45]; float ke[576]; };

struct LaunchCtx {
    cudaStream_t stream;
    Scalars* S;
    RedBuf rb;
    int tma = 0;  // bit 0: FP32 2x restrictions with TMA-staged rows; bit 1: bulk-staged mixed prolongation
};

// Opt the matvec kernels into > 48 KB of dynamic shared memory (once per device).
cudaError_t setKernelAttributes();

// ---- launchers (return the number of kernels launched) ----
template <typename T>
int launchMatvec(const LaunchCtx& c, const MatvecArgs<T>& a, bool structured, const void* opconst);

// The same product on FP64 vectors in double-float arithmetic (FP32 instructions,
// ~48-bit significands): the mixed-precision true residual.  a.y may be null.
int launchMatvecDF(const LaunchCtx& c, const MatvecArgs<double>& a, bool structured, const double* opconst);

// checkDone: 1 = skip once the solve is done; 2 = also skip unless the true
// residual replaced r in this iteration (2x coarsening only).
template <typename T>
int launchRestrict(const LaunchCtx& c, const Grid& gf, const Grid& gc, int div, const T* rf, T* rc,
                   int checkDone);

// Reference-mode up-leg: zf = used ? P zc + coef * dinv o rf : 0 (fixed -> 0 on level 0),
// optional dots r.z and z.aux with epilogue `epi`.  hd (FP32, 2x coarsening):
// the inverse diagonal as FP16 values times a power of two, read instead of dinv.
struct HalfDiag {
    const __half* d = nullptr;
    float scale = 1.0f;
};
template <typename T>
int launchProlongSmooth(const LaunchCtx& c, const Grid& gf, const Grid& gc, int div, const T* zc, const T* rf,
                        const T* dinv, const uint8_t* flags, T* zf, double coef, int maskFixed,
                        const T* aux, int epi, int checkDone, HalfDiag hd = HalfDiag());

// V-cycle helpers: z = mask(omega dinv r); zf += mask(P zc).
template <typename T>
int launchJacobiZero(const LaunchCtx& c, const Grid& g, const T* r, const T* dinv, const uint8_t* flags, T* z,
                     double omega, int checkDone);
template <typename T>
int launchProlongAdd(const LaunchCtx& c, const Grid& gf, const Grid& gc, int div, const T* zc,
                     const uint8_t* flags, T* zf, int checkDone);

// Coarsest level: zc[free] = Kinv * rc[free].  FP32 (the mixed-precision
// cycle): Kinv is the packed lower block triangle of CT x CT tiles stored in
// FP16 (launchPackSymHalf), value = scale * stored; tmp holds coarseBlocks(n) * CT
// values (zero past n), part 2 * CT values per tile.  FP64: Kinv is the full
// n x n matrix (part unused).
constexpr int CT = 64;
inline int64_t coarseBlocks(int64_t n) { return (n + CT - 1) / CT; }
inline int64_t coarseTiles(int64_t n) { return coarseBlocks(n) * (coarseBlocks(n) + 1) / 2; }
template <typename T>
struct CoarseInv;
template <>
struct CoarseInv<double> {
    const double* K;
};
template <>
struct CoarseInv<float> {
    const __half* K;
    float scale;
};
template <typename T>
int launchCoarseSolve(const LaunchCtx& c, CoarseInv<T> Kinv, int64_t n, const int32_t* freeDof, const T* rc, T* tmp,
                      T* part, T* zc, int checkDone);
// *outBits = max |x_i| as FP32 bits (zero *outBits first); y = FP16(x * invScale).
int launchMaxAbs(cudaStream_t s, const float* x, int64_t n, unsigned* outBits);
int launchToHalf(cudaStream_t s, const float* x, int64_t n, float invScale, __half* y);
// *out = the largest diagonal entry of a row-major n x n matrix.
int launchMaxDiag(cudaStream_t s, const float* K, int64_t n, float* out);
// Pack a full symmetric row-major n x n matrix, times invScale, into
// coarseTiles(n) FP16 tiles.
int launchPackSymHalf(cudaStream_t s, const float* K, int64_t n, float invScale, __half* tiles);

// CG vector updates on flat arrays of length n.
// x += alpha p ; r -= alpha Ap ; rr -> EPI_CONV (FP64 solver: TX = TV = double)
template <typename TX, typename TV>
int launchUpdateXR(const LaunchCtx& c, int64_t n, TX* x, TV* r, const TV* p, const TV* Ap);
// x64 += x32 (+ the deferred alpha p); x32 = 0 (mixed precision).  conditional:
// only in iterations that recompute the FP64 true residual.
int launchFlushX(const LaunchCtx& c, int64_t n, double* x64, float* x32, const float* p, const float* pAlt,
                 int conditional);
// FP32 CG product with the direction update fused into its input stage
// (structured Ke): p = z + beta p_old, x32 += alpha p_old (unless folded),
// y = K p (fixed rows 0), p.(Kp) -> EPI_ALPHA; flips Scalars::pSel.
int launchMatvecPX(const LaunchCtx& c, const MatvecArgs<float>& a, const float* opconst);
// Mixed precision: r -= alpha Ap with r.r (x += alpha p deferred); p = z + beta p
// with the deferred x += alpha p.
int launchUpdateR(const LaunchCtx& c, int64_t n, float* r, const float* Ap);
int launchUpdatePX(const LaunchCtx& c, int64_t n, float* p, const float* z, float* x);
// Mixed precision, reference cycle with a 2x first coarsening: the residual
// update fused with the first restriction (rOut = rIn - alpha Ap, r.r, rc =
// R rOut); rOut must not alias rIn.
int launchUpdateRestrict(const LaunchCtx& c, const Grid& gf, const Grid& gc, const float* rIn, const float* Ap,
                         float* rOut, float* rc);
// p = z + beta p
template <typename T>
int launchUpdateP(const LaunchCtx& c, int64_t n, T* p, const T* z, int first);
// sums (a.b, c.d) -> epi  (pointers may alias; null pair -> 0)
template <typename T>
int launchDots(const LaunchCtx& c, int64_t n, const T* a, const T* b, const T* cc, const T* d, int epi,
               int checkDone);
// y = x (with type conversion), optional x2 -> y2 zero fill
template <typename TI, typename TO>
int launchConvert(cudaStream_t s, int64_t n, const TI* x, TO* y);
template <typename T>
int launchFill(cudaStream_t s, int64_t n, T* y, T v);

// compressed <-> dense storage
template <typename T>
// comp may be host memory when the device reads pageable memory directly; bad
// (optional) gets bit 0 set when comp holds a non-finite value.
int launchScatterCompressed(cudaStream_t s, int64_t nnodes, const int32_t* nodeStore, const double* comp, T* dense,
                            unsigned* bad = nullptr);
template <typename T>
int launchGatherCompressed(cudaStream_t s, int64_t nnodes, const int32_t* nodeStore, const T* dense, double* comp);

// Coarsest-matrix assembly (dense, free DOFs only), one parity colour per launch.
template <typename T>
int launchAssembleCoarse(cudaStream_t s, const Grid& g, const float* E, const int32_t* freeNode, const double* Ke,
                         double scale, T* K, int64_t n);
template <typename T>
int launchSymmetrizeLowerToFull(cudaStream_t s, T* K, int64_t n);
// Zero the strict lower triangle of a row-major n x n matrix (cuSOLVER's
// column-major upper triangle).
template <typename T>
int launchZeroStrictRowMajorLower(cudaStream_t s, T* K, int64_t n);

// Deflated preconditioner (A-DEF2 of Tang, Nabben, Vuik and Erlangga, J. Sci.
// Comput. 39 (2009)): z <- z + V G^-1 (V^T r - (KV)^T z) for z = M^-1 r; two
// kernels, the 2k dots with G^-1 applied by the last block, then the update.
template <typename T>
int launchCoarseSpace(const LaunchCtx& c, int64_t n, int k, const T* V, const T* KV, const CoarseSpace& G,
                      const T* r, T* z, int checkDone);
// Start projection of deflated CG: x <- x + V mu, r <- r - KV mu, mu = G^-1 V^T r.
int launchCoarseStart(const LaunchCtx& c, int64_t n, int k, const double* V, const double* KV, const CoarseSpace& G,
                      double* x, double* r);

// Solver scalar initialisation (device side, so it can live in a graph).
int launchInitScalars(cudaStream_t s, Scalars* S, double tol, long long maxIter, int flexible, int mixed,
                      int replaceEvery, double replaceDelta, int breakAt = 0);

// FP64 product y = K x with the fused x.(Kx) dot, its reduction scratch taken from
// a file-scope device array (kernels.cu) instead of allocated memory.  The first
// call on a device looks up that array's device address.  *tooLarge is set (and
// nothing launched) when the product's grid needs more reduction blocks than
// the array holds.  xKx is a device pointer.
cudaError_t launchMatvecNoAlloc(cudaStream_t s, const MatvecArgs<double>& a, bool structured, const void* opconst,
                                double* xKx, bool* tooLarge);

// Tensor-core FP32 CG product (matvec_tc.cu): B = q Ke in BF16 as K-major core
// matrices, invScale = 1 / q.  tcPrepare fails (false) when no integer
// q <= 65536 makes every entry of q Ke an integer exact in BF16.
struct alignas(16) TcOperand {
    uint32_t b[512];
    float invScale;
    int q;
};
bool tcPrepare(const double* Ke, TcOperand& out);
// The product form the tensor-core kernel computes: y = K x (fixed rows 0) and x.(Kx).
bool tcEligible(const MatvecArgs<float>& a);
cudaError_t tcSetAttributes();
int launchMatvecTC(const LaunchCtx& c, const MatvecArgs<float>& a, const TcOperand& op);
int64_t tcBlocks(const Grid& g);  // reduction blocks of a launch

// FP32 2x restriction with TMA-staged fine rows (transfer_tma.cu); Ap != null:
// with the fused residual update (rOut = rIn - alpha Ap, r.r).  Returns 0 (and
// launches nothing) when a tensor map cannot be made for the vectors.
cudaError_t tmaSetAttributes();
bool tmaAvailable(const float* v, int64_t n);  // a tensor map can be made for these n floats
// The mixed V-cycle's 2x up-leg (kProlongFlat<float, __half> semantics) with its
// ranges staged by bulk copies; the vectors must come from allocations with at
// least 16 spare bytes past their end.  Returns 0 (nothing launched) for grids
// whose ranges exceed the shared-memory budget.
int launchProlongBulk(const LaunchCtx& c, const Grid& gf, const Grid& gc, const float* zc, const float* rf,
                      const __half* dinv, const uint8_t* flags, float* zf, double coef, int maskFixed,
                      const float* aux, int epi, int checkDone);
int launchRestrictTma(const LaunchCtx& c, const Grid& gf, const Grid& gc, const float* rIn, const float* Ap,
                      float* rOut, float* rc, int checkDone);

// Device-side ``done`` / iteration snapshot is read back by the host with a plain copy.

}  // namespace vfem
