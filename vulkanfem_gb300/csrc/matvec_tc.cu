// matvec_tc.cu -- the FP32 CG product y = K x on the 5th-generation tensor cores
// (tcgen05.mma, accumulators in tensor memory), sm_103a.
//
// Replaces MatxVec.comp + FixedNodes.comp + VecDotVec.comp of the reference
// (include/MatrixFreeSparse.hpp:197-214: y += Ke x_e per element, fixed rows
// zeroed; the CG's p.Ap) for the mixed-precision solve's product.  Opt-in
// (VFEM_TENSOR_CORE_PRODUCT=1 when the problem is created): on GB300 it is
// correct to FP32 accuracy but slower than the Walsh-factorised CUDA-core
// kernel (kMatvecH), because every MMA of this shape is bound by reading its A
// operand from shared memory (an M = 128, N = 32, K = 16 BF16 MMA takes ~28 ns,
// the same as N = 64; about 1/8 of the tensor pipe's peak rate), and the three
// BF16 terms need 24 such MMAs per 512 elements.
//
// The element product as a GEMM.  Element e's 24 input values (8 corners x 3
// components) form one row of A, and D = A B^T with B = q Ke, where q is an
// integer scale that makes every entry of q Ke an integer exactly representable
// in BF16 (q = 1872 for the 2x2x2-Gauss hex at nu = 0.3, largest entry 440);
// y_e = (E_e scale / q) D_e.  Node values are split into three BF16 terms,
// x = h + m + l up to 2^-27 |x|, so the three BF16 products, accumulated in FP32
// in tensor memory, give the product to FP32 accuracy.
//
// Operand A without gathering.  A corner slot holds 4 BF16 values (x, y, z, 0),
// and the "pair record" of node n holds the slots of n and of its +x neighbour
// (16 bytes).  The record of an element's lower corner is then the element's
// corners 0 and 1 (a = dx + 2 dy + 4 dz, K index 4a + c), the record one node row
// up its corners 2 and 3, and the records of the next node layer corners 4..7.
// With records stored row by row, 8 elements consecutive in x have consecutive
// records, which is exactly the no-swizzle K-major core matrix (8 rows of 16
// bytes): one MMA (M = 128, N = 32, K = 16) reads 8 x 16 elements of a layer
// straight from the node tile, with the K-direction core-matrix stride (LBO)
// and the M-direction one (SBO) both equal to one record row.  The 4th value of
// every slot is zero, so K = 32 and N = 32 hold the 24 inputs and outputs.
//
// Tile and pipeline.  A CTA of 256 threads owns 31 x 15 node columns and marches
// TC_ZC node layers up z; per element layer it computes the 32 x 16 elements
// whose corners touch its nodes (4 MMAs of 128 elements x 3 terms x 2 K steps,
// issued by one thread, committed to an mbarrier).  Tensor memory holds two
// accumulator buffers (2 x 4 x 32 columns), so the MMAs of layer k run while
// the threads read back layer k-1: each thread takes two elements (its TMEM
// lane), scales them by E_e scale / q, folds the top-face outputs of the layer
// below (kept in registers, as the Walsh-carry kernel does) into the bottom-face
// ones, and exchanges three corner sums through shared memory so that the
// owner of each node adds its four in-layer contributions: no atomics, fixed
// summation order, deterministic.  Node values are loaded into registers two
// layers ahead, then split and written as records into a 2-layer ring (the
// layer an MMA batch reads is overwritten only after its mbarrier completes).
// Every wait is bounded: a wait that runs out sets the solve's BREAKDOWN and
// timeout flags, the CTA skips its remaining tensor work, still joins the grid
// reduction, and frees its tensor memory.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>

#include "kernels.h"
#include "reduce.cuh"

namespace vfem {

namespace {

constexpr int TC_EX = 32, TC_EY = 16;            // elements per layer of a CTA tile
constexpr int TC_ZC = 32;                         // node layers owned per CTA
constexpr int TC_NT = 256;                        // threads per CTA
constexpr int TC_ROW_B = TC_EX * 16;              // one row of pair records (bytes)
constexpr int TC_TERM_B = (TC_EY + 1) * TC_ROW_B; // records of one term of a node layer
constexpr int TC_LAYER_B = 3 * TC_TERM_B;         // hi, mid, lo terms
constexpr int TC_B_OFF = 2 * TC_LAYER_B;          // B tile (2048 bytes) after the 2-layer ring
constexpr int TC_XR_OFF = TC_B_OFF + 2048;        // FP32 x of the owned-position nodes, 4-layer ring
constexpr int TC_XR_LAYER = TC_EX * TC_EY * 3 * 4;
constexpr int TC_XB_OFF = TC_XR_OFF + 4 * TC_XR_LAYER;  // corner-sum exchange, 512 elements x 3 x 16 B
constexpr int TC_SMEM = TC_XB_OFF + TC_EX * TC_EY * 3 * 16;
constexpr uint32_t TC_TMEM_COLS = 256;            // 2 accumulator buffers x 4 MMAs x N = 32
constexpr long long TC_WAIT_LIMIT = 1ll << 22;    // mbarrier polls before a wait gives up
// kind::f16 instruction descriptor: D F32 (bits 4-5 = 1), A and B BF16 (bits 7-9,
// 10-12 = 1), both K-major, N = 32 (bits 17-22 = N >> 3), M = 128 (bits 24-28 = M >> 4).
constexpr uint32_t TC_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ uint32_t smemAddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor, no swizzle: start address, leading (K-direction)
// and stride (M/N-direction) byte offsets between core matrices, version 1 (bit 46).
__device__ __forceinline__ uint64_t tcDesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ void tcMma(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t accum) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
        "l"(ad), "l"(bd), "r"(TC_IDESC), "r"(accum));
}

// 16 consecutive FP32 accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tcLd16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Bounded wait for the completion of mbarrier phase `parity`; false if it ran out.
__device__ __forceinline__ bool mbarWait(uint32_t mbar, uint32_t parity) {
    for (long long it = 0; it < TC_WAIT_LIMIT; ++it) {
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

// Three BF16 terms of a pair of FP32 values, each packed as a bf16x2 word.
__device__ __forceinline__ float2 unpackBf2(uint32_t u) {
    return make_float2(__uint_as_float(u << 16), __uint_as_float(u & 0xffff0000u));
}
__device__ __forceinline__ uint32_t packBf2(float2 v) {
    const __nv_bfloat162 b = __floats2bfloat162_rn(v.x, v.y);
    return *reinterpret_cast<const uint32_t*>(&b);
}
__device__ __forceinline__ void split3(float2 v, uint32_t (&t)[3]) {
    t[0] = packBf2(v);
    const float2 r1 = __ffma2_rn(unpackBf2(t[0]), make_float2(-1.f, -1.f), v);  // exact: v - RN(v)
    t[1] = packBf2(r1);
    const float2 r2 = __ffma2_rn(unpackBf2(t[1]), make_float2(-1.f, -1.f), r1);
    t[2] = packBf2(r2);
}

// Register bundle loaded two element layers ahead: the staged nodes' values
// (two owned-position nodes and, in threads 0..48, one halo node), the moduli
// of the thread's two elements and the flags of their owned nodes.
struct TcBundle {
    float x[3][3];
    float E[2];
    uint32_t fl[2];
};

__global__ void __launch_bounds__(TC_NT, 2)
    kMatvecTC(MatvecArgs<float> a, const __grid_constant__ TcOperand op, Scalars* S, RedBuf rb) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tslot;
    __shared__ int sflag;
    const int tid = threadIdx.x;
    if (tid == 0) sflag = (a.checkDone && S->done) ? 1 : 0;
    __syncthreads();
    if (sflag) return;  // uniform: read once by one thread

    const int w = tid >> 5, lane = tid & 31, wq = w & 3, jh = w >> 2;
    const int gnx = a.g.nx, gny = a.g.ny, gnz = a.g.nz;
    const int ex0 = blockIdx.x * (TC_EX - 1) - 1, ey0 = blockIdx.y * (TC_EY - 1) - 1;
    const int z0 = blockIdx.z * TC_ZC, zend = min(z0 + TC_ZC, gnz);
    const int64_t plane = (int64_t)gnx * gny;

    // The thread's two elements (TMEM lane 32 wq + lane of MMAs j = 2 jh, 2 jh + 1):
    // local (lx0 + 8 jj, ly); their owned nodes, local (lx + 1, ly + 1), are also
    // the nodes the thread stages, plus one halo node (row 0, or column 0 below
    // row 1) in threads 0..48.
    const int ly = 4 * wq + (lane >> 3);
    const int lx0 = 16 * jh + (lane & 7);
    const int ncol = (ey0 + ly + 1) * gnx + ex0 + lx0 + 1;  // grid column of the first staged node
    const int hx = tid < 33 ? tid : 0, hy = tid < 33 ? 0 : tid - 32;
    const int hcol = (ey0 + hy) * gnx + ex0 + hx;
    unsigned m = 0;  // validity bits: staged nodes 0-2, elements 3-4, owned nodes 5-6
    {
        const int gy = ey0 + ly + 1;
#pragma unroll
        for (int jj = 0; jj < 2; ++jj) {
            const int gx = ex0 + lx0 + 8 * jj + 1;
            if (gx >= 0 && gx < gnx && gy >= 0 && gy < gny) m |= 1u << jj;
            if (gx - 1 >= 0 && gx - 1 < a.g.ex && gy - 1 >= 0 && gy - 1 < a.g.ey) m |= 8u << jj;
            if (lx0 + 8 * jj < TC_EX - 1 && ly < TC_EY - 1 && gx < gnx && gy < gny) m |= 32u << jj;
        }
        const int gx = ex0 + hx, gyh = ey0 + hy;
        if (tid < 49 && gx >= 0 && gx < gnx && gyh >= 0 && gyh < gny) m |= 4u;
    }

    auto loadBundle = [&](TcBundle& b, int xLayer, int eLayer) {
        const int64_t xo = (int64_t)xLayer * plane, eo = (int64_t)eLayer * plane;
        const bool xz = xLayer >= 0 && xLayer < gnz;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const bool ok = xz && (m & (1u << q));
            const float* p = a.x + 3 * ((q < 2 ? (int64_t)(ncol + 8 * q) : (int64_t)hcol) + xo);
#pragma unroll
            for (int c = 0; c < 3; ++c) b.x[q][c] = ok ? __ldg(p + c) : 0.f;
        }
        const bool ez = eLayer >= 0 && eLayer < a.g.ez, fz = eLayer >= z0 && eLayer < zend;
#pragma unroll
        for (int jj = 0; jj < 2; ++jj) {
            const int64_t c = (int64_t)(ncol + 8 * jj) + eo;
            b.E[jj] = (ez && (m & (8u << jj))) ? __ldg(a.E + c - gnx - 1) : 0.f;
            b.fl[jj] = (fz && (m & (32u << jj))) ? (uint32_t)__ldg(a.flags + c) : 0u;
        }
    };
    // Records of node layer L (values in b.x) into ring slot L & 1, and the FP32
    // values of the owned-position nodes into the x ring (slot (L + 4) % 4; L >= -1).
    // The x ring has 4 slots: layer L + 3 is staged in the iteration whose
    // read-back reads layer L, with no barrier in between.
    auto stage = [&](const TcBundle& b, int L) {
        unsigned char* ring = sm + (L & 1) * TC_LAYER_B;
        float* xr = reinterpret_cast<float*>(sm + TC_XR_OFF + ((L + 4) & 3) * TC_XR_LAYER) + 3 * (ly * TC_EX + lx0);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            if (q == 2 && tid >= 49) break;
            uint32_t txy[3], tz[3];
            split3(make_float2(b.x[q][0], b.x[q][1]), txy);
            split3(make_float2(b.x[q][2], 0.f), tz);
            const int nx = q < 2 ? lx0 + 8 * q + 1 : hx, ny = q < 2 ? ly + 1 : hy;
            unsigned char* row = ring + ny * TC_ROW_B + nx * 16;
#pragma unroll
            for (int t = 0; t < 3; ++t) {
                const uint2 slot = make_uint2(txy[t], tz[t]);
                if (nx < TC_EX) *reinterpret_cast<uint2*>(row + t * TC_TERM_B) = slot;
                if (nx > 0) *reinterpret_cast<uint2*>(row + t * TC_TERM_B - 8) = slot;
            }
            if (q < 2) {
                xr[24 * q] = b.x[q][0];
                xr[24 * q + 1] = b.x[q][1];
                xr[24 * q + 2] = b.x[q][2];
            }
        }
    };

    // ---- set-up: B tile, mbarrier, tensor memory, the first two node layers
    {
        const uint4* src = reinterpret_cast<const uint4*>(op.b);
        uint4* dst = reinterpret_cast<uint4*>(sm + TC_B_OFF);
        if (tid < 128) dst[tid] = src[tid];
    }
    const uint32_t mb = smemAddr(&mbar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (w == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(&tslot)),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    TcBundle b0, b1;
    loadBundle(b0, z0 - 1, -1);
    stage(b0, z0 - 1);
    loadBundle(b1, z0, -1);
    stage(b1, z0);
    // b0 feeds iteration 0 (stages node layer z0 + 1); b1 feeds iteration 1
    // (stages z0 + 2; reads back element layer z0 - 1).
    loadBundle(b0, z0 + 1, -1);
    loadBundle(b1, z0 + 2, z0 - 1);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tbase = tslot;
    const uint32_t smb = smemAddr(sm);

    float carry[2][12];
#pragma unroll
    for (int jj = 0; jj < 2; ++jj)
#pragma unroll
        for (int i = 0; i < 12; ++i) carry[jj][i] = 0.f;
    double dAx = 0.0;
    bool bad = false;
    float4* xb = reinterpret_cast<float4*>(sm + TC_XB_OFF);
    const float cs = a.scale * op.invScale;

    // Read-back of element layer e (accumulator buffer buf): combine with the
    // carried top faces, exchange, and write node layer e when it is owned.
    auto epilogue = [&](const TcBundle& b, int e, int buf) {
        float own[2][3];
#pragma unroll
        for (int jj = 0; jj < 2; ++jj) {
            const uint32_t ta = tbase + ((uint32_t)(32 * wq) << 16) + (uint32_t)(buf * 128 + 32 * (2 * jh + jj));
            const float s = b.E[jj] * cs;
            float d[16];
            if (!bad) tcLd16(ta, d);
            else {
#pragma unroll
                for (int i = 0; i < 16; ++i) d[i] = 0.f;
            }
            float4* slot = xb + 3 * (ly * TC_EX + lx0 + 8 * jj);
#pragma unroll
            for (int cn = 0; cn < 4; ++cn) {
                float v[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) v[c] = fmaf(s, d[4 * cn + c], carry[jj][3 * cn + c]);
                if (cn < 3) slot[cn] = make_float4(v[0], v[1], v[2], 0.f);  // corners (0,0), (1,0), (0,1)
                else {
                    own[jj][0] = v[0];                                       // corner (1,1): the owned node
                    own[jj][1] = v[1];
                    own[jj][2] = v[2];
                }
            }
            if (!bad) tcLd16(ta + 16, d);
#pragma unroll
            for (int cn = 0; cn < 4; ++cn)
#pragma unroll
                for (int c = 0; c < 3; ++c) carry[jj][3 * cn + c] = s * d[4 * cn + c];
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        if (e >= z0) {
            const float* xr = reinterpret_cast<const float*>(sm + TC_XR_OFF + ((e + 4) & 3) * TC_XR_LAYER);
            const int64_t lo = (int64_t)e * plane;
            float dl = 0.f;  // this layer's x.(Kx) terms (at most 6), added to the FP64 sum
#pragma unroll
            for (int jj = 0; jj < 2; ++jj) {
                if (!(m & (32u << jj))) continue;
                const int el = ly * TC_EX + lx0 + 8 * jj;
                const float4 r = xb[3 * (el + 1) + 2];            // element (x+1, y): its corner (0,1)
                const float4 u = xb[3 * (el + TC_EX) + 1];        // element (x, y+1): its corner (1,0)
                const float4 v = xb[3 * (el + TC_EX + 1) + 0];    // element (x+1, y+1): its corner (0,0)
                const bool fixed = (b.fl[jj] & FLAG_FIXED) != 0;
                float* y = a.y + 3 * ((int64_t)(ncol + 8 * jj) + lo);
                const float* xo = xr + 3 * el;
                const float o0 = fixed ? 0.f : own[jj][0] + r.x + u.x + v.x;
                const float o1 = fixed ? 0.f : own[jj][1] + r.y + u.y + v.y;
                const float o2 = fixed ? 0.f : own[jj][2] + r.z + u.z + v.z;
                y[0] = o0;
                y[1] = o1;
                y[2] = o2;
                dl = fmaf(xo[0], o0, dl);
                dl = fmaf(xo[1], o1, dl);
                dl = fmaf(xo[2], o2, dl);
            }
            dAx += (double)dl;
        }
    };

    const int nIter = zend - z0 + 1;  // element layers z0 - 1 .. zend - 1
    auto iteration = [&](TcBundle& b, int i) {
        const int k = z0 - 1 + i;
        // (1) MMAs of element layer k: node layers k (ring slot k & 1) and k + 1.
        if (tid == 0 && !bad) {
            const uint32_t s0 = smb + (uint32_t)((k & 1) * TC_LAYER_B);
            const uint32_t s1 = smb + (uint32_t)(((k + 1) & 1) * TC_LAYER_B);
            const uint32_t bb = smb + TC_B_OFF;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint32_t dt = tbase + (uint32_t)((i & 1) * 128 + 32 * j);
#pragma unroll
                for (int t = 0; t < 3; ++t) {
                    tcMma(dt, tcDesc(s0 + t * TC_TERM_B + 128 * j, TC_ROW_B, TC_ROW_B), tcDesc(bb, 128, 512),
                          t > 0 ? 1u : 0u);
                    tcMma(dt, tcDesc(s1 + t * TC_TERM_B + 128 * j, TC_ROW_B, TC_ROW_B), tcDesc(bb + 256, 128, 512),
                          1u);
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mb)
                         : "memory");
        }
        // (2) read-back of element layer k - 1 (buffer (i - 1) & 1, complete)
        if (i > 0) epilogue(b, k - 1, (i - 1) & 1);
        // (3) wait for this layer's MMAs; then node layer k + 2 replaces layer k
        const bool ok = bad || mbarWait(mb, (uint32_t)(i & 1));
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        stage(b, k + 2);
        loadBundle(b, k + 4, k + 1);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        if (__syncthreads_or(!ok)) bad = true;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    };
    int i = 0;
    for (; i + 1 < nIter; i += 2) {
        iteration(b0, i);
        iteration(b1, i + 1);
    }
    if (i < nIter) {
        iteration(b0, i);
        epilogue(b1, zend - 1, (nIter - 1) & 1);
    } else {
        epilogue(b0, zend - 1, (nIter - 1) & 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (w == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(TC_TMEM_COLS)
                     : "memory");
    }
    if (bad && tid == 0) {
        S->kernelTimeout = 1;
        S->done = BREAKDOWN;
    }
    if (a.epi != EPI_NONE) {
        double v[2] = {dAx, 0.0}, t[2];
        if (gridReduce<TC_NT, 2>(v, rb, t)) applyEpi(a.epi, S, t[0], t[1]);
    }
}

// bf16 bits of an exactly representable value
uint16_t bf16Bits(double v) {
    float f = (float)v;
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return (uint16_t)(u >> 16);
}

}  // namespace

bool tcPrepare(const double* Ke, TcOperand& out) {
    double mx = 0.0;
    for (int i = 0; i < 576; ++i) mx = std::fmax(mx, std::fabs(Ke[i]));
    if (!(mx > 0.0) || !std::isfinite(mx)) return false;
    // the smallest integer q with q Ke integer-valued and every entry exact in BF16
    int q = 0;
    for (int cand = 1; cand <= 65536 && !q; ++cand) {
        bool okAll = true;
        for (int i = 0; i < 576 && okAll; ++i) {
            const double v = cand * Ke[i], r = std::nearbyint(v);
            if (std::fabs(v - r) > 1e-9 * cand * mx) okAll = false;
            else if (r != 0.0) {
                // at most 8 significant bits
                int e = 0;
                std::frexp(r, &e);
                const double mnt = std::ldexp(std::fabs(r), 8 - e);
                if (mnt != std::floor(mnt)) okAll = false;
            }
        }
        if (okAll) q = cand;
    }
    if (!q) return false;
    std::memset(out.b, 0, sizeof(out.b));
    uint16_t* b = reinterpret_cast<uint16_t*>(out.b);
    // B[n][k] = q Ke[3 bo + co][3 ai + ci] for n = 4 bo + co, k = 4 ai + ci (0 on the 4th slot values),
    // K-major no-swizzle core matrices: (n / 8, k / 8) at (n / 8) 512 + (k / 8) 128 bytes, row n % 8 at
    // 16 bytes, k % 8 at 2 bytes.
    for (int n = 0; n < 32; ++n)
        for (int k = 0; k < 32; ++k) {
            const int bo = n / 4, co = n % 4, ai = k / 4, ci = k % 4;
            const double v = (co < 3 && ci < 3) ? std::nearbyint(q * Ke[(3 * bo + co) * 24 + 3 * ai + ci]) : 0.0;
            b[((n / 8) * 512 + (k / 8) * 128 + (n % 8) * 16 + (k % 8) * 2) / 2] = bf16Bits(v);
        }
    out.invScale = (float)(1.0 / q);
    out.q = q;
    return true;
}

bool tcEligible(const MatvecArgs<float>& a) {
    return a.mode == MV_AX && a.dot0 == DOT_X_OUT && !a.dot1 && !a.y32 && !a.condTrue;
}

cudaError_t tcSetAttributes() {
    return cudaFuncSetAttribute(kMatvecTC, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
}

int launchMatvecTC(const LaunchCtx& c, const MatvecArgs<float>& a, const TcOperand& op) {
    const Grid& g = a.g;
    dim3 grid((g.nx + TC_EX - 2) / (TC_EX - 1), (g.ny + TC_EY - 2) / (TC_EY - 1), (g.nz + TC_ZC - 1) / TC_ZC);
    kMatvecTC<<<grid, TC_NT, TC_SMEM, c.stream>>>(a, op, c.S, c.rb);
    return 1;
}

int64_t tcBlocks(const Grid& g) {
    return (int64_t)((g.nx + TC_EX - 2) / (TC_EX - 1)) * ((g.ny + TC_EY - 2) / (TC_EY - 1)) *
           ((g.nz + TC_ZC - 1) / TC_ZC);
}

}  // namespace vfem
