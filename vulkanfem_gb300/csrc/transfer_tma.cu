// transfer_tma.cu -- FP32 multigrid transfers with TMA-staged fine rows, sm_103a.
//
// kRestrictTma replaces CWiseMult.comp + Restrict.comp (and, fused, the residual
// update of ConjugateGradient_1.comp) of the reference
// (include/MultigridPreconditioner.hpp:67-108) for the 2x coarsening in FP32:
// rc[C] = sum_{|d| <= 1} prod_i (1 - |d_i| / 2) r[2C + d] on the dense grids, the
// reference's W-weighted per-element restriction in its structured form.  With
// UPD it first forms the updated residual r - alpha Ap, writes it for the fine
// nodes a coarse cell owns (fine x, y, z in {2c, 2c + 1}) and sums its squares
// for r.r, exactly as kRestrict2<float, true> does.
//
// Data movement.  Vectors hold 3 floats per node (12-byte nodes), so a thread
// that owns coarse column cx and reads fine nodes 2cx - 1 .. 2cx + 1 straight
// from global memory issues loads 24 bytes apart across the warp (several L1
// wavefronts per request).  Here a CTA (32 x 8 coarse columns, 4 coarse layers)
// stages every fine row segment it needs -- 65 nodes, 195 floats -- into shared
// memory with one TMA tile load (`cp.async.bulk.tensor.1d`) per row and vector,
// through a 1-D tensor map over the whole vector: the row's start is rounded
// down to a 16-byte boundary (the TMA rule for the innermost coordinate) and
// the box of 224 floats (896 bytes, keeping every shared-memory destination
// 128-byte aligned, as TMA tile loads require) covers the rest; coordinates before the start or past
// the end of the vector read zeros.  Rows outside the grid are not loaded, and
// fine nodes outside the grid are masked, as in kRestrict2.  Fine planes go
// through a ring of 3 (fused update) or 4 plane slots, each with an mbarrier that counts the
// transaction bytes of its TMA loads; one thread issues the loads of the next
// planes as soon as every thread has finished with the planes they replace
// (one CTA barrier per coarse layer), so about two coarse layers of loads are
// in flight.  Every wait is bounded: a wait that runs out sets the solve's
// BREAKDOWN and timeout flags, and the CTA still joins the grid reduction.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdlib>
#include <cstring>
#include <mutex>
#include <type_traits>

#include "kernels.h"
#include "reduce.cuh"

namespace vfem {

namespace {

constexpr int RT_CX = 32, RT_CZ = 4;  // coarse cells per CTA in x and z (CY in y: a template parameter)
// floats per row load: >= 195 + 3 alignment floats, and 896 bytes, a multiple of
// 128, because a TMA tile load's shared-memory destination must be 128-byte aligned
constexpr int RT_BOX = 224;
constexpr int RT_ROW_B = RT_BOX * 4;
static_assert(RT_ROW_B % 128 == 0, "TMA destinations must stay 128-byte aligned");
// plane slots: 3 with the fused update (two vectors; 91 KB, two CTAs per SM), 4 without (61 KB)
template <bool UPD>
__host__ __device__ constexpr int rtSlots() { return UPD ? 3 : 4; }
template <bool UPD, int CY>
__host__ __device__ constexpr int rtSmem() { return rtSlots<UPD>() * (UPD ? 2 : 1) * (2 * CY + 1) * RT_ROW_B; }
constexpr long long RT_WAIT_LIMIT = 1ll << 22;

__device__ __forceinline__ uint32_t smemAddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool mbarWait(uint32_t mbar, uint32_t parity) {
    for (long long it = 0; it < RT_WAIT_LIMIT; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tmaLoad1d(uint32_t dst, const CUtensorMap* map, int c0, uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.tensor.1d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2}], [%3];" ::"r"(
            dst),
        "l"(map), "r"(c0), "r"(mbar)
        : "memory");
}

// floor to a multiple of 4 (the TMA start of a row: 16 bytes of floats)
__device__ __forceinline__ int64_t floor4(int64_t v) { return v >= 0 ? (v & ~(int64_t)3) : -((-v + 3) & ~(int64_t)3); }

template <bool UPD, int CY>
__global__ void __launch_bounds__(32 * CY) kRestrictTma(const __grid_constant__ CUtensorMap mapR,
                                                    const __grid_constant__ CUtensorMap mapA, Grid gf, Grid gc,
                                                    float* __restrict__ rOut, float* __restrict__ rc, Scalars* S,
                                                    RedBuf rb, int checkDone) {
    constexpr int RT_SLOTS = rtSlots<UPD>();
    constexpr int RT_ROWS = 2 * CY + 1;  // fine rows per plane
    __shared__ int sflag;
    __shared__ __align__(8) uint64_t bar[RT_SLOTS];
    extern __shared__ __align__(128) unsigned char rtSmem[];
    constexpr int NV = UPD ? 2 : 1;
    const int lane = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + lane;
    if (tid == 0) sflag = (checkDone && S->done) || (checkDone == 2 && S->replStamp != S->matvecs);
    __syncthreads();
    if (sflag) return;
    const int cx0 = blockIdx.x * RT_CX, cy0 = blockIdx.y * CY, cz0 = blockIdx.z * RT_CZ;
    const int nl = min(RT_CZ, gc.nz - cz0);  // coarse layers of this CTA
    const int np = 2 * nl + 1;              // fine planes 2 cz0 - 1 .. 2 (cz0 + nl) - 1
    const int64_t fplane = (int64_t)gf.nx * gf.ny;
    const uint32_t sbase = smemAddr(rtSmem);
    // Issue the TMA loads of local plane p into its slot (one thread).
    auto issue = [&](int p) {
        const int fz = 2 * cz0 - 1 + p, slot = p % RT_SLOTS;
        const uint32_t mb = smemAddr(&bar[slot]);
        uint32_t rows = 0;
        if (fz >= 0 && fz < gf.nz)
            for (int lr = 0; lr < RT_ROWS; ++lr) {
                const int fy = 2 * cy0 - 1 + lr;
                rows += (fy >= 0 && fy < gf.ny) ? 1u : 0u;
            }
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(rows * NV * RT_ROW_B)
                     : "memory");
        if (!rows) return;
        for (int lr = 0; lr < RT_ROWS; ++lr) {
            const int fy = 2 * cy0 - 1 + lr;
            if (fy < 0 || fy >= gf.ny) continue;
            const int64_t start = 3 * ((int64_t)fz * fplane + (int64_t)fy * gf.nx + 2 * cx0 - 1);
            const int c0 = (int)floor4(start);
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                const uint32_t dst = sbase + (uint32_t)(((slot * NV + v) * RT_ROWS + lr) * RT_ROW_B);
                tmaLoad1d(dst, v ? &mapA : &mapR, c0, mb);
            }
        }
    };
    if (tid == 0) {
        for (int s = 0; s < RT_SLOTS; ++s)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smemAddr(&bar[s])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        for (int p = 0; p < min(np, RT_SLOTS); ++p) issue(p);
    }
    __syncthreads();
    int issued = min(np, RT_SLOTS);

    const int cx = cx0 + lane, cy = cy0 + ty;
    const bool valid = cx < gc.nx && cy < gc.ny;
    const float av = UPD ? (float)S->alpha : 0.f;
    DotAcc<float> acc;
    bool timedOut = false;
    // Weighted sum of local plane p at this thread's coarse column (fine rows
    // 2cy - 1 .. 2cy + 1, each r(2cx - 1)/2 + r(2cx) + r(2cx + 1)/2); with UPD the
    // owned fine nodes of an owned plane are updated, written and summed.
    auto planeSum = [&](int p, bool ownPlane, float (&P)[3]) {
        const int fz = 2 * cz0 - 1 + p, slot = p % RT_SLOTS;
        if (!mbarWait(smemAddr(&bar[slot]), (uint32_t)((p / RT_SLOTS) & 1))) timedOut = true;
        const bool zok = fz >= 0 && fz < gf.nz;
        float row[3][3];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            const int lr = 2 * ty + r, fy = 2 * cy0 - 1 + lr;
            const bool rowOk = zok && fy >= 0 && fy < gf.ny && !timedOut;
            const int64_t start = 3 * ((int64_t)fz * fplane + (int64_t)fy * gf.nx + 2 * cx0 - 1);
            const int o = (int)(start - floor4(start));
            const float* rp = reinterpret_cast<const float*>(rtSmem + ((slot * NV) * RT_ROWS + lr) * RT_ROW_B) + o;
            const float* ap =
                reinterpret_cast<const float*>(rtSmem + ((slot * NV + NV - 1) * RT_ROWS + lr) * RT_ROW_B) + o;
            float v[3][3];
            bool okd[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const int lx = 2 * lane + d, fx = 2 * cx0 - 1 + lx;
                const bool ok = rowOk && fx >= 0 && fx < gf.nx;
                okd[d] = ok;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    float x = ok ? rp[3 * lx + c] : 0.f;
                    if (UPD) x = ok ? fmaf(-av, ap[3 * lx + c], x) : 0.f;
                    v[d][c] = x;
                }
            }
            if (UPD && ownPlane && valid && r >= 1) {
                // the owned fine nodes 2cx, 2cx + 1 of this row, summed in kRestrict2's order
                float* q = rOut + 3 * ((int64_t)fz * fplane + (int64_t)fy * gf.nx + 2 * cx0 + 2 * lane);
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    if (okd[1]) {
                        q[c] = v[1][c];
                        acc.add(v[1][c] * v[1][c]);
                    }
                    if (okd[2]) {
                        q[3 + c] = v[2][c];
                        acc.add(v[2][c] * v[2][c]);
                    }
                }
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) row[r][c] = v[1][c] + 0.5f * (v[0][c] + v[2][c]);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) P[c] = row[1][c] + 0.5f * (row[0][c] + row[2][c]);
    };
    float Pm[3];
    planeSum(0, false, Pm);
    for (int l = 0; l < nl; ++l) {
        const int cz = cz0 + l;
        float P0[3], Pp[3];
        planeSum(2 * l + 1, true, P0);
        planeSum(2 * l + 2, true, Pp);
        if (valid) {
            float* q = rc + 3 * gc.store(cx, cy, cz);
#pragma unroll
            for (int c = 0; c < 3; ++c) q[c] = P0[c] + 0.5f * (Pm[c] + Pp[c]);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) Pm[c] = Pp[c];
        // planes <= 2l + 2 are consumed: their slots take the next planes
        const int upto = 2 * l + 3 + RT_SLOTS;
        if (issued < np && issued < upto) {
            __syncthreads();
            if (tid == 0) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                for (int p = issued; p < np && p < upto; ++p) issue(p);
            }
            issued = min(np, upto);
        }
    }
    if (timedOut) {
        S->kernelTimeout = 1;
        S->done = BREAKDOWN;
    }
    if (UPD) {
        double v[1] = {acc.get()}, t[1];
        if (gridReduce<32 * CY, 1>(v, rb, t)) applyEpi(EPI_CONV, S, t[0], 0.0);
    }
}

// ---------------------------------------------------------------- prolongation
//
// kProlongBulk: the 2x up-leg of the mixed V-cycle (kProlongFlat<float, __half>:
// zf = used ? P zc + coef dinv o rf : 0, fixed rows zeroed on the finest level,
// r.z and z.aux), with its inputs staged by the bulk-copy engine.  A block owns
// fine rows [fy0, fy0 + 16) of one fine layer, which are one contiguous range of
// every fine vector, and the (up to) 9 coarse rows they interpolate from, which
// are contiguous in each coarse layer.  One thread issues one `cp.async.bulk`
// per range (r, the FP16 inverse diagonal, the flags, one or two coarse layers;
// each range widened to 16-byte boundaries, which the allocations' 64 spare
// bytes keep in bounds) on one mbarrier; the threads then compute from shared
// memory in kProlongFlat's node order and arithmetic (so the result and the dots
// are bit-identical), write z over r in shared memory, and store the block's
// range of z with consecutive threads on consecutive floats.

__device__ __forceinline__ void bulkLoad(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
}

struct PbLayout {  // byte offsets of the staged ranges (16-byte aligned)
    int c1, c2, r, d, f, total;
};
__host__ __device__ inline int pbAlign(int64_t b) { return (int)((b + 15) & ~(int64_t)15); }
__host__ __device__ inline PbLayout pbLayout(const Grid& gf, const Grid& gc, int rows) {
    PbLayout L;
    const int cspan = pbAlign((int64_t)(rows / 2 + 1) * 3 * gc.nx * 4 + 32);
    const int64_t nbMax = (int64_t)rows * gf.nx;
    L.c1 = 0;
    L.c2 = cspan;
    L.r = 2 * cspan;
    L.d = L.r + pbAlign(12 * nbMax + 32);
    L.f = L.d + pbAlign(6 * nbMax + 32);
    L.total = L.f + pbAlign(nbMax + 32);
    return L;
}

__global__ void __launch_bounds__(256)
    kProlongBulk(Grid gf, Grid gc, const float* __restrict__ zc, const float* __restrict__ rf,
                 const __half* __restrict__ dinv, const uint8_t* __restrict__ flags, float* __restrict__ zf, float cf,
                 int maskFixed, const float* __restrict__ aux, int epi, float invNx, Scalars* S, RedBuf rb,
                 int checkDone, int rows) {
    if (checkDone && S->done) return;
    extern __shared__ __align__(128) unsigned char pbSmem[];
    __shared__ __align__(8) uint64_t bar;
    const int tid = threadIdx.x;
    const PbLayout Lo = pbLayout(gf, gc, rows);
    const int groups = (gf.ny + rows - 1) / rows;
    const int fz = blockIdx.x / groups;
    const int fy0 = (blockIdx.x - fz * groups) * rows, fy1 = min(gf.ny, fy0 + rows);
    const int cw = 3 * gc.nx, cy0 = fy0 >> 1, cz = fz >> 1;
    const int nstage = min(rows / 2 + 1, gc.ny - cy0) * cw;
    const bool zodd = fz & 1;
    const int64_t nBeg = gf.store(0, fy0, fz);
    const int nb = (fy1 - fy0) * gf.nx;
    const int64_t nEnd = nBeg + nb;
    // aligned byte ranges and the element offset of each range's first wanted value
    const int64_t cb = 4 * (3 * gc.store(0, cy0, cz)), cb2 = cb + 4 * 3 * ((int64_t)gc.nx * gc.ny);
    const int64_t ca = cb & ~(int64_t)15, ca2 = cb2 & ~(int64_t)15;
    const int64_t ra = (12 * nBeg) & ~(int64_t)15, da = (6 * nBeg) & ~(int64_t)15, fa = nBeg & ~(int64_t)15;
    const uint32_t mb = (uint32_t)__cvta_generic_to_shared(&bar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        const uint32_t sb = (uint32_t)__cvta_generic_to_shared(pbSmem);
        const uint32_t nc = (uint32_t)(((cb + 4 * (int64_t)nstage + 15) & ~(int64_t)15) - ca);
        const uint32_t nc2 = (uint32_t)(((cb2 + 4 * (int64_t)nstage + 15) & ~(int64_t)15) - ca2);
        const uint32_t nr = (uint32_t)(((12 * nEnd + 15) & ~(int64_t)15) - ra);
        const uint32_t nd = (uint32_t)(((6 * nEnd + 15) & ~(int64_t)15) - da);
        const uint32_t nf = (uint32_t)(((nEnd + 15) & ~(int64_t)15) - fa);
        const uint32_t tx = nc + (zodd ? nc2 : 0u) + nr + nd + nf;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(tx) : "memory");
        const char* zcb = reinterpret_cast<const char*>(zc);
        bulkLoad(sb + Lo.c1, zcb + ca, nc, mb);
        if (zodd) bulkLoad(sb + Lo.c2, zcb + ca2, nc2, mb);
        bulkLoad(sb + Lo.r, reinterpret_cast<const char*>(rf) + ra, nr, mb);
        bulkLoad(sb + Lo.d, reinterpret_cast<const char*>(dinv) + da, nd, mb);
        bulkLoad(sb + Lo.f, reinterpret_cast<const char*>(flags) + fa, nf, mb);
    }
    __syncthreads();
    bool ok = mbarWait(mb, 0);
    float* C = reinterpret_cast<float*>(pbSmem + Lo.c1 + (cb - ca));
    if (zodd) {
        const float* C2 = reinterpret_cast<const float*>(pbSmem + Lo.c2 + (cb2 - ca2));
        for (int q = tid; q < nstage; q += 256) C[q] = 0.5f * (C[q] + C2[q]);
    }
    if (__syncthreads_or(!ok)) {
        if (tid == 0) {
            S->kernelTimeout = 1;
            S->done = BREAKDOWN;
        }
    }
    float* R = reinterpret_cast<float*>(pbSmem + Lo.r + (12 * nBeg - ra)) - 3 * nBeg;  // R[3 n + c], n in the range
    const __half* Dh = reinterpret_cast<const __half*>(pbSmem + Lo.d + (6 * nBeg - da)) - 3 * nBeg;
    const uint8_t* F = reinterpret_cast<const uint8_t*>(pbSmem + Lo.f + (nBeg - fa)) - nBeg;
    const float half = 0.5f;
    DotAcc<float> d0, d1;
    const int64_t j1 = (nEnd + 3) >> 2;
    for (int64_t j = (nBeg >> 2) + tid; j < j1; j += 256) {
        const int64_t n0 = 4 * j;
        const int ln0 = (int)(n0 - nBeg);
        const int lnc = max(ln0, 0);
        int ly = __float2int_rz(((float)lnc + 0.5f) * invNx);
        int fx = lnc - ly * gf.nx;
        if (fx < 0) { --ly; fx += gf.nx; }
        if (fx >= gf.nx) { ++ly; fx -= gf.nx; }
        fx -= lnc - ln0;
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int ln = ln0 + t;
            if (ln >= 0 && ln < nb) {
                const int64_t n = n0 + t;
                const uint32_t fl = F[n];
                const bool used = (fl & FLAG_USED) != 0;
                const bool zero = !used || (maskFixed && (fl & FLAG_FIXED));
                const float* b = C + (ly >> 1) * cw + 3 * (fx >> 1);
                float pv[3];
                if (fx & 1) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) pv[c] = half * (b[c] + b[c + 3]);
                } else {
#pragma unroll
                    for (int c = 0; c < 3; ++c) pv[c] = b[c];
                }
                if (ly & 1) {
                    const float* b1 = b + cw;
                    if (fx & 1) {
#pragma unroll
                        for (int c = 0; c < 3; ++c) pv[c] = half * (pv[c] + half * (b1[c] + b1[c + 3]));
                    } else {
#pragma unroll
                        for (int c = 0; c < 3; ++c) pv[c] = half * (pv[c] + b1[c]);
                    }
                }
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float r = used ? R[3 * n + c] : 0.f;
                    const float out = zero ? 0.f : pv[c] + cf * __half2float(Dh[3 * n + c]) * r;
                    if (epi != EPI_NONE) {
                        d0.add(r * out);
                        if (aux) d1.add(out * aux[3 * n + c]);
                    }
                    R[3 * n + c] = out;  // z replaces r (this thread's nodes only)
                }
            }
            if (++fx == gf.nx) {
                fx = 0;
                ++ly;
            }
        }
    }
    __syncthreads();
    for (int64_t i = 3 * nBeg + tid; i < 3 * nEnd; i += 256) zf[i] = R[i];
    if (epi != EPI_NONE) {
        double v[2] = {d0.get(), d1.get()}, t[2];
        if (gridReduce<256, 2>(v, rb, t)) applyEpi(epi, S, t[0], t[1]);
    }
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encodeOnce;

// 1-D tensor map over n floats at ptr, boxes of RT_BOX floats, zero fill out of range.
bool encode1d(CUtensorMap* m, const float* ptr, int64_t n) {
    std::call_once(g_encodeOnce, [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    });
    if (!g_encode || !ptr || n <= 0 || n >= (int64_t(1) << 32) || (reinterpret_cast<uintptr_t>(ptr) & 15u)) return false;
    const cuuint64_t dim[1] = {(cuuint64_t)n};
    const cuuint64_t stride[1] = {(cuuint64_t)n * 4};  // unused for rank 1, but the encoder rejects a null array
    const cuuint32_t box[1] = {(cuuint32_t)RT_BOX};
    const cuuint32_t es[1] = {1};
    return g_encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 1, const_cast<float*>(ptr), dim, stride, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

bool tmaAvailable(const float* v, int64_t n) {
    CUtensorMap m;
    return encode1d(&m, v, n);
}

cudaError_t tmaSetAttributes() {
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(kRestrictTma<true, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  rtSmem<true, 8>())) != cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(kRestrictTma<false, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  rtSmem<false, 8>())) != cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(kRestrictTma<true, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  rtSmem<true, 4>())) != cudaSuccess)
        return e;
    return cudaFuncSetAttribute(kRestrictTma<false, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                rtSmem<false, 4>());
}

int launchProlongBulk(const LaunchCtx& c, const Grid& gf, const Grid& gc, const float* zc, const float* rf,
                      const __half* dinv, const uint8_t* flags, float* zf, double coef, int maskFixed,
                      const float* aux, int epi, int checkDone) {
    static const int rows = [] {
        const char* v = std::getenv("VFEM_PB_ROWS");
        const int r = v ? std::atoi(v) : 8;
        return (r >= 2 && r <= 32 && r % 2 == 0) ? r : 8;
    }();
    const PbLayout L = pbLayout(gf, gc, rows);
    const int64_t blocks = (int64_t)((gf.ny + rows - 1) / rows) * gf.nz;
    if (L.total > 200 * 1024 || blocks > kMaxRedBlocks) return 0;
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(kProlongBulk, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) !=
            cudaSuccess)
            return 0;
        attr = true;
    }
    kProlongBulk<<<(unsigned)blocks, 256, L.total, c.stream>>>(gf, gc, zc, rf, dinv, flags, zf, (float)coef, maskFixed,
                                                               aux, epi, 1.0f / gf.nx, c.S, c.rb, checkDone, rows);
    return 1;
}

int launchRestrictTma(const LaunchCtx& c, const Grid& gf, const Grid& gc, const float* rIn, const float* Ap,
                      float* rOut, float* rc, int checkDone) {
    CUtensorMap mr, ma;
    const int64_t n = 3 * gf.nnode;
    if (!encode1d(&mr, rIn, n)) return 0;
    if (Ap) {
        if (!encode1d(&ma, Ap, n)) return 0;
    } else {
        ma = mr;
    }
    static const int cy = [] {
        const char* v = std::getenv("VFEM_RT_CY");
        return (v && std::atoi(v) == 8) ? 8 : 4;
    }();
    auto go = [&](auto cyTag) {
        constexpr int CY = decltype(cyTag)::value;
        dim3 block(32, CY), grid((gc.nx + RT_CX - 1) / RT_CX, (gc.ny + CY - 1) / CY, (gc.nz + RT_CZ - 1) / RT_CZ);
        if (Ap)
            kRestrictTma<true, CY><<<grid, block, rtSmem<true, CY>(), c.stream>>>(mr, ma, gf, gc, rOut, rc, c.S, c.rb,
                                                                                  checkDone);
        else
            kRestrictTma<false, CY><<<grid, block, rtSmem<false, CY>(), c.stream>>>(mr, ma, gf, gc, nullptr, rc, c.S,
                                                                                    c.rb, checkDone);
    };
    if (cy == 8) go(std::integral_constant<int, 8>());
    else go(std::integral_constant<int, 4>());
    return 1;
}

}  // namespace vfem
