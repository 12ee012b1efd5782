// unet.cu -- the learned part of the solver: a small 3-D U-Net on the node grid
// (inputs: occupancy, modulus, fixed mask, load; output: displacement), trained
// and run with this file's own kernels.  No reference counterpart.
//
// Numerics: activations and weights in BF16, every product accumulated in FP32
// on the tensor cores (mma.sync m16n8k16 bf16 -> f32), FP32 master weights and
// Adam moments.  Layout: channels-last [voxel][channel] on an n^3 grid (n a
// multiple of 8), x fastest.
//
// Network (4 levels, 16-32-64-128 channels; every conv is 3x3x3, zero padded):
//   e0 = relu(conv(x, 16->16))        @ n      p1 = avgpool2(e0)
//   e1 = relu(conv(p1, 16->32))       @ n/2    p2 = avgpool2(e1)
//   e2 = relu(conv(p2, 32->64))       @ n/4    p3 = avgpool2(e2)
//   e3 = relu(conv(p3, 64->128))      @ n/8
//   d2 = relu(conv([up2(e3), e2], 192->64))  @ n/4
//   d1 = relu(conv([up2(d2), e1],  96->32))  @ n/2
//   d0 = relu(conv([up2(d1), e0],  48->16))  @ n
//   y  = conv(d0, 16->16)  (channels 0..2 are the prediction)
// Kernels: kConvFwd (implicit GEMM; also the data gradient with flipped,
// transposed weights), kConvWGrad (weight gradient, split over voxels), pooling,
// nearest upsampling, concat/split, ReLU mask, bias gradient, masked MSE, Adam.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "vfem_net.h"

namespace {

thread_local std::string g_netError;

constexpr int kLayers = 8;
// (Cin, Cout, level, relu) of the 8 convolutions.
constexpr int kCin[kLayers] = {16, 16, 32, 64, 192, 96, 48, 16};
constexpr int kCout[kLayers] = {16, 32, 64, 128, 64, 32, 16, 16};
constexpr int kLevel[kLayers] = {0, 1, 2, 3, 2, 1, 0, 0};
constexpr int kRelu[kLayers] = {1, 1, 1, 1, 1, 1, 1, 0};

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ uint32_t pack2(bf16 lo, bf16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ void mma16816(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// ----------------------------------------------------------------------------- convolution
// Implicit GEMM: out[v][co] = sum_{tap, ci} in[v + off(tap)][ci] * W[tap][ci][co] (+ bias, relu).
// Block: 128 threads (4 warps) computes 64 consecutive voxels x 64 output channels
// (or Cout if smaller).  K loop over 27 taps x Cin/16 chunks; A (64 x 16) and B
// (16 x 64) staged in shared memory; each warp owns 16 voxel rows.
constexpr int CT_M = 64, CT_N = 64, CT_K = 16;

template <bool OUT_F32>
__global__ void __launch_bounds__(128) kConvFwd(const bf16* __restrict__ in, const bf16* __restrict__ W,
                                                const float* __restrict__ bias, void* __restrict__ out, int n, int Cin,
                                                int Cout, int relu) {
    __shared__ __align__(16) bf16 sA[CT_M][CT_K + 8];   // +8: break bank conflicts
    __shared__ __align__(16) bf16 sB[CT_K][CT_N + 8];
    __shared__ int sxyz[CT_M][3];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t V = (int64_t)n * n * n;
    const int64_t v0 = (int64_t)blockIdx.x * CT_M;
    const int n0 = blockIdx.y * CT_N;
    const int nt = min(CT_N, Cout - n0);  // multiple of 16
    if (tid < CT_M) {
        const int64_t v = v0 + tid;
        sxyz[tid][0] = (int)(v % n);
        sxyz[tid][1] = (int)((v / n) % n);
        sxyz[tid][2] = (int)(v / ((int64_t)n * n));
    }
    float acc[CT_N / 8][4];
#pragma unroll
    for (int j = 0; j < CT_N / 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    __syncthreads();
    const int g = lane >> 2, t4 = lane & 3;
    for (int tap = 0; tap < 27; ++tap) {
        const int dx = tap % 3 - 1, dy = (tap / 3) % 3 - 1, dz = tap / 9 - 1;
        for (int c0 = 0; c0 < Cin; c0 += CT_K) {
            // A: 64 voxels x 16 channels, one 8-channel half per thread.
            {
                const int r = tid >> 1, h = tid & 1;
                const int x = sxyz[r][0] + dx, y = sxyz[r][1] + dy, z = sxyz[r][2] + dz;
                uint4 val = make_uint4(0, 0, 0, 0);
                if (v0 + r < V && x >= 0 && x < n && y >= 0 && y < n && z >= 0 && z < n) {
                    const int64_t src = ((int64_t)z * n + y) * n + x;
                    val = *reinterpret_cast<const uint4*>(in + src * Cin + c0 + 8 * h);
                }
                *reinterpret_cast<uint4*>(&sA[r][8 * h]) = val;
            }
            // B: 16 input channels x nt output channels.
            for (int i = tid; i < CT_K * (nt / 8); i += 128) {
                const int k = i / (nt / 8), q = i % (nt / 8);
                *reinterpret_cast<uint4*>(&sB[k][8 * q]) =
                    *reinterpret_cast<const uint4*>(W + ((int64_t)tap * Cin + c0 + k) * Cout + n0 + 8 * q);
            }
            __syncthreads();
            const int rb = warp * 16;
            const uint32_t a0 = pack2(sA[rb + g][2 * t4], sA[rb + g][2 * t4 + 1]);
            const uint32_t a1 = pack2(sA[rb + g + 8][2 * t4], sA[rb + g + 8][2 * t4 + 1]);
            const uint32_t a2 = pack2(sA[rb + g][2 * t4 + 8], sA[rb + g][2 * t4 + 9]);
            const uint32_t a3 = pack2(sA[rb + g + 8][2 * t4 + 8], sA[rb + g + 8][2 * t4 + 9]);
#pragma unroll
            for (int j = 0; j < CT_N / 8; ++j) {
                if (8 * j >= nt) break;
                const uint32_t b0 = pack2(sB[2 * t4][8 * j + g], sB[2 * t4 + 1][8 * j + g]);
                const uint32_t b1 = pack2(sB[2 * t4 + 8][8 * j + g], sB[2 * t4 + 9][8 * j + g]);
                mma16816(acc[j], a0, a1, a2, a3, b0, b1);
            }
            __syncthreads();
        }
    }
    const int rb = warp * 16;
#pragma unroll
    for (int j = 0; j < CT_N / 8; ++j) {
        if (8 * j >= nt) break;
#pragma unroll
        for (int hrow = 0; hrow < 2; ++hrow) {
            const int64_t v = v0 + rb + g + 8 * hrow;
            if (v >= V) continue;
            const int co = n0 + 8 * j + 2 * t4;
            float y0 = acc[j][2 * hrow] + (bias ? bias[co] : 0.f);
            float y1 = acc[j][2 * hrow + 1] + (bias ? bias[co + 1] : 0.f);
            if (relu) {
                y0 = fmaxf(y0, 0.f);
                y1 = fmaxf(y1, 0.f);
            }
            if (OUT_F32) {
                float* o = static_cast<float*>(out) + v * Cout + co;
                o[0] = y0;
                o[1] = y1;
            } else {
                bf16* o = static_cast<bf16*>(out) + v * Cout + co;
                o[0] = __float2bfloat16(y0);
                o[1] = __float2bfloat16(y1);
            }
        }
    }
}

// Weight gradient: dW[tap][ci][co] += sum_v in[v + off(tap)][ci] * g[v][co].
// Grid (voxel chunks, taps, ci tiles x co tiles); block 128 threads computes a
// 64(ci) x 64(co) tile over its voxel chunk in steps of 16 voxels and stores it
// in the chunk's slice of part ([chunk][27][Cin][Cout]); kWGradSum then adds
// the chunks to dW in a fixed order, so the gradient is bit-reproducible.
constexpr int WG_CHUNK = 2048;

__global__ void __launch_bounds__(128) kConvWGrad(const bf16* __restrict__ in, const bf16* __restrict__ gout,
                                                  float* __restrict__ part, int n, int Cin, int Cout) {
    __shared__ __align__(16) bf16 sA[64][16 + 8];   // [ci][v]
    __shared__ __align__(16) bf16 sB[16][64 + 8];   // [v][co]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g = lane >> 2, t4 = lane & 3;
    const int tap = blockIdx.y;
    const int dx = tap % 3 - 1, dy = (tap / 3) % 3 - 1, dz = tap / 9 - 1;
    const int ciTiles = (Cin + 63) / 64;
    const int ci0 = (blockIdx.z % ciTiles) * 64, co0 = (blockIdx.z / ciTiles) * 64;
    const int mt = min(64, Cin - ci0), nt = min(64, Cout - co0);
    const int64_t V = (int64_t)n * n * n;
    const int64_t vb = (int64_t)blockIdx.x * WG_CHUNK;
    const int64_t ve = min(V, vb + WG_CHUNK);
    float acc[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    for (int64_t vs = vb; vs < ve; vs += 16) {
        // A^T tile: 16 voxels x mt channels of the shifted input.
        for (int i = tid; i < 16 * (mt / 8); i += 128) {
            const int vv = i / (mt / 8), q = i % (mt / 8);
            const int64_t v = vs + vv;
            uint4 val = make_uint4(0, 0, 0, 0);
            if (v < ve) {
                const int x = (int)(v % n) + dx, y = (int)((v / n) % n) + dy, z = (int)(v / ((int64_t)n * n)) + dz;
                if (x >= 0 && x < n && y >= 0 && y < n && z >= 0 && z < n)
                    val = *reinterpret_cast<const uint4*>(in + (((int64_t)z * n + y) * n + x) * Cin + ci0 + 8 * q);
            }
            const bf16* e = reinterpret_cast<const bf16*>(&val);
#pragma unroll
            for (int u = 0; u < 8; ++u) sA[8 * q + u][vv] = e[u];
        }
        for (int i = tid; i < 16 * (nt / 8); i += 128) {
            const int vv = i / (nt / 8), q = i % (nt / 8);
            const int64_t v = vs + vv;
            uint4 val = make_uint4(0, 0, 0, 0);
            if (v < ve) val = *reinterpret_cast<const uint4*>(gout + v * Cout + co0 + 8 * q);
            *reinterpret_cast<uint4*>(&sB[vv][8 * q]) = val;
        }
        __syncthreads();
        const int rb = warp * 16;
        if (rb < mt) {
            const uint32_t a0 = pack2(sA[rb + g][2 * t4], sA[rb + g][2 * t4 + 1]);
            const uint32_t a1 = pack2(sA[rb + g + 8][2 * t4], sA[rb + g + 8][2 * t4 + 1]);
            const uint32_t a2 = pack2(sA[rb + g][2 * t4 + 8], sA[rb + g][2 * t4 + 9]);
            const uint32_t a3 = pack2(sA[rb + g + 8][2 * t4 + 8], sA[rb + g + 8][2 * t4 + 9]);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                if (8 * j >= nt) break;
                const uint32_t b0 = pack2(sB[2 * t4][8 * j + g], sB[2 * t4 + 1][8 * j + g]);
                const uint32_t b1 = pack2(sB[2 * t4 + 8][8 * j + g], sB[2 * t4 + 9][8 * j + g]);
                mma16816(acc[j], a0, a1, a2, a3, b0, b1);
            }
        }
        __syncthreads();
    }
    const int rb = warp * 16;
    if (rb >= mt) return;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        if (8 * j >= nt) break;
#pragma unroll
        for (int hrow = 0; hrow < 2; ++hrow) {
            const int ci = ci0 + rb + g + 8 * hrow;
            const int co = co0 + 8 * j + 2 * t4;
            float* d = part + (int64_t)blockIdx.x * 27 * Cin * Cout + ((int64_t)tap * Cin + ci) * Cout + co;
            d[0] = acc[j][2 * hrow];
            d[1] = acc[j][2 * hrow + 1];
        }
    }
}

// dW[e] += sum over chunks c (in order) of part[c][e], e < per (= 27 Cin Cout).
__global__ void kWGradSum(const float* __restrict__ part, float* __restrict__ dW, int64_t per, int chunks) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < per; e += (int64_t)gridDim.x * blockDim.x) {
        float sum = 0.f;
        for (int c = 0; c < chunks; ++c) sum += part[(int64_t)c * per + e];
        dW[e] += sum;
    }
}

// ----------------------------------------------------------------------------- elementwise
__global__ void kPool(const bf16* __restrict__ in, bf16* __restrict__ out, int nc, int C) {
    // out at n/2 = nc: mean of the 2x2x2 children.
    const int64_t total = (int64_t)nc * nc * nc * C;
    const int nf = 2 * nc;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const int64_t v = i / C;
        const int x = (int)(v % nc), y = (int)((v / nc) % nc), z = (int)(v / ((int64_t)nc * nc));
        float s = 0.f;
#pragma unroll
        for (int d = 0; d < 8; ++d) {
            const int X = 2 * x + (d & 1), Y = 2 * y + ((d >> 1) & 1), Z = 2 * z + (d >> 2);
            s += __bfloat162float(in[(((int64_t)Z * nf + Y) * nf + X) * C + c]);
        }
        out[i] = __float2bfloat16(0.125f * s);
    }
}

// d(in) = d(out)/8 broadcast to the children (avg-pool backward); accumulate = 1 adds.
__global__ void kPoolBwd(const float* __restrict__ gout, float* __restrict__ gin, int nc, int C, int accumulate) {
    const int nf = 2 * nc;
    const int64_t total = (int64_t)nf * nf * nf * C;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const int64_t v = i / C;
        const int x = (int)(v % nf) / 2, y = (int)((v / nf) % nf) / 2, z = (int)(v / ((int64_t)nf * nf)) / 2;
        const float gv = 0.125f * gout[(((int64_t)z * nc + y) * nc + x) * C + c];
        gin[i] = accumulate ? gin[i] + gv : gv;
    }
}

// Decoder input: channels [0, Ca) = nearest upsampling of a (at n/2), [Ca, Ca+Cb) = skip b.
__global__ void kUpConcat(const bf16* __restrict__ a, const bf16* __restrict__ b, bf16* __restrict__ out, int nf,
                          int Ca, int Cb) {
    const int C = Ca + Cb, nc = nf / 2;
    const int64_t total = (int64_t)nf * nf * nf * C;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const int64_t v = i / C;
        if (c < Ca) {
            const int x = (int)(v % nf) / 2, y = (int)((v / nf) % nf) / 2, z = (int)(v / ((int64_t)nf * nf)) / 2;
            out[i] = a[(((int64_t)z * nc + y) * nc + x) * Ca + c];
        } else {
            out[i] = b[v * Cb + (c - Ca)];
        }
    }
}

// Backward of kUpConcat: ga (at n/2) = sum of the 8 children's first Ca channels,
// gb (skip) = the remaining channels (added to an existing gradient).
__global__ void kUpConcatBwd(const float* __restrict__ g, float* __restrict__ ga, float* __restrict__ gb, int nf,
                             int Ca, int Cb) {
    const int C = Ca + Cb, nc = nf / 2;
    const int64_t totalA = (int64_t)nc * nc * nc * Ca;
    const int64_t totalB = (int64_t)nf * nf * nf * Cb;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < totalA + totalB;
         i += (int64_t)gridDim.x * blockDim.x) {
        if (i < totalA) {
            const int c = (int)(i % Ca);
            const int64_t v = i / Ca;
            const int x = (int)(v % nc), y = (int)((v / nc) % nc), z = (int)(v / ((int64_t)nc * nc));
            float s = 0.f;
#pragma unroll
            for (int d = 0; d < 8; ++d) {
                const int X = 2 * x + (d & 1), Y = 2 * y + ((d >> 1) & 1), Z = 2 * z + (d >> 2);
                s += g[(((int64_t)Z * nf + Y) * nf + X) * C + c];
            }
            ga[i] = s;
        } else {
            const int64_t j = i - totalA;
            const int c = (int)(j % Cb);
            const int64_t v = j / Cb;
            gb[j] += g[v * C + Ca + c];
        }
    }
}

// Gradient through relu: gmask = g * (y > 0) as bf16 (operand of the backward GEMMs).
__global__ void kReluMask(const float* __restrict__ g, const bf16* __restrict__ y, bf16* __restrict__ out, int64_t n,
                          int relu) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = __float2bfloat16((!relu || __bfloat162float(y[i]) > 0.f) ? g[i] : 0.f);
}

__global__ void kBiasGrad(const bf16* __restrict__ g, float* __restrict__ db, int64_t V, int C) {
    // One block per channel group of 32 channels; threads stride over voxels.
    __shared__ float s[256];
    const int c = blockIdx.x;
    float acc = 0.f;
    for (int64_t v = threadIdx.x; v < V; v += blockDim.x) acc += __bfloat162float(g[v * C + c]);
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[c] += s[0];
}

// Masked MSE on channels 0..2 of y (C channels): loss = sum m (y - t)^2 / count;
// grad written to gy (all C channels, 0 beyond 2).  partial sums in part[blockIdx].
__global__ void kMse(const float* __restrict__ y, const float* __restrict__ t, const float* __restrict__ m,
                     float* __restrict__ gy, double* __restrict__ part, int64_t V, int C, float invCount) {
    __shared__ double s[256];
    double acc = 0.0;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
        const float mv = m[v];
        for (int c = 0; c < C; ++c) {
            float gr = 0.f;
            if (c < 3) {
                const float d = y[v * C + c] - t[v * 3 + c];
                acc += (double)(mv * d * d);
                gr = 2.f * mv * d * invCount;
            }
            gy[v * C + c] = gr;
        }
    }
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

__global__ void kAdam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                      int64_t n, float lr, float b1, float b2, float eps, float c1, float c2, float gscale) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i] * gscale;
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

// Working BF16 weights from the FP32 master: W (as is) and Wt[26 - tap][co][ci] for
// the data gradient.
__global__ void kCastWeights(const float* __restrict__ w, bf16* __restrict__ wb, bf16* __restrict__ wt, int Cin,
                             int Cout) {
    const int64_t n = 27LL * Cin * Cout;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int co = (int)(i % Cout);
        const int ci = (int)((i / Cout) % Cin);
        const int tap = (int)(i / ((int64_t)Cin * Cout));
        const bf16 b = __float2bfloat16(w[i]);
        wb[i] = b;
        wt[((int64_t)(26 - tap) * Cout + co) * Cin + ci] = b;
    }
}

__global__ void kF32ToBf16(const float* __restrict__ x, bf16* __restrict__ y, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = __float2bfloat16(x[i]);
}

inline int blocks(int64_t n) {
    int64_t b = (n + 255) / 256;
    return (int)(b > 4096 ? 4096 : (b < 1 ? 1 : b));
}

}  // namespace

// ----------------------------------------------------------------------------- network object
struct vfem_net {
    int n = 0;  // finest grid size (multiple of 8)
    int64_t V[4] = {};
    cudaStream_t stream = nullptr;
    // parameters: per layer weights [27][Cin][Cout] then bias [Cout], packed FP32
    int64_t woff[kLayers] = {}, boff[kLayers] = {}, nparam = 0;
    float *w = nullptr, *gw = nullptr, *m = nullptr, *v = nullptr;
    bf16 *wb[kLayers] = {}, *wt[kLayers] = {};
    int64_t step = 0;
    // activations (bf16) and gradients (f32)
    bf16 *x = nullptr, *e[4] = {}, *p[4] = {}, *c[3] = {}, *d[3] = {};
    float* y = nullptr;
    float *t = nullptr, *mask = nullptr, *gy = nullptr;
    float *ge[4] = {}, *gp[4] = {}, *gc[3] = {}, *gd[3] = {};
    bf16* gmask = nullptr;  // masked gradient scratch (largest layer)
    bf16* gbf = nullptr;    // bf16 copy of an input gradient (largest)
    float* wgPart = nullptr;  // per-chunk weight-gradient tiles (largest layer)
    double* part = nullptr;
    float* hostStage = nullptr;
};

namespace {

vfem_status netFail(vfem_status s, const std::string& m) {
    g_netError = m;
    return s;
}

#define NCK(call)                                                                                    \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) return netFail(VFEM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Zeroed device allocation, complete on return (the memset runs on the legacy
// default stream, which the network's non-blocking stream does not wait for).
template <typename T>
cudaError_t nalloc(T** p, int64_t n) {
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * (size_t)(n > 0 ? n : 1));
    if (e != cudaSuccess) return e;
    e = cudaMemset(*p, 0, sizeof(T) * (size_t)(n > 0 ? n : 1));
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(cudaStreamLegacy);
}

void conv(vfem_net* N, const bf16* in, const bf16* W, const float* b, void* out, int lvl, int Cin, int Cout, int relu,
          bool f32) {
    const int n = N->n >> lvl;
    dim3 grid((unsigned)((N->V[lvl] + CT_M - 1) / CT_M), (unsigned)((Cout + CT_N - 1) / CT_N));
    if (f32) kConvFwd<true><<<grid, 128, 0, N->stream>>>(in, W, b, out, n, Cin, Cout, relu);
    else kConvFwd<false><<<grid, 128, 0, N->stream>>>(in, W, b, out, n, Cin, Cout, relu);
}

void forward(vfem_net* N) {
    const int64_t* V = N->V;
    for (int l = 0; l < kLayers; ++l)
        kCastWeights<<<blocks(27LL * kCin[l] * kCout[l]), 256, 0, N->stream>>>(N->w + N->woff[l], N->wb[l], N->wt[l],
                                                                                 kCin[l], kCout[l]);
    auto B = [&](int l) { return N->w + N->boff[l]; };
    conv(N, N->x, N->wb[0], B(0), N->e[0], 0, 16, 16, 1, false);
    kPool<<<blocks(V[1] * 16), 256, 0, N->stream>>>(N->e[0], N->p[1], N->n / 2, 16);
    conv(N, N->p[1], N->wb[1], B(1), N->e[1], 1, 16, 32, 1, false);
    kPool<<<blocks(V[2] * 32), 256, 0, N->stream>>>(N->e[1], N->p[2], N->n / 4, 32);
    conv(N, N->p[2], N->wb[2], B(2), N->e[2], 2, 32, 64, 1, false);
    kPool<<<blocks(V[3] * 64), 256, 0, N->stream>>>(N->e[2], N->p[3], N->n / 8, 64);
    conv(N, N->p[3], N->wb[3], B(3), N->e[3], 3, 64, 128, 1, false);
    kUpConcat<<<blocks(V[2] * 192), 256, 0, N->stream>>>(N->e[3], N->e[2], N->c[2], N->n / 4, 128, 64);
    conv(N, N->c[2], N->wb[4], B(4), N->d[2], 2, 192, 64, 1, false);
    kUpConcat<<<blocks(V[1] * 96), 256, 0, N->stream>>>(N->d[2], N->e[1], N->c[1], N->n / 2, 64, 32);
    conv(N, N->c[1], N->wb[5], B(5), N->d[1], 1, 96, 32, 1, false);
    kUpConcat<<<blocks(V[0] * 48), 256, 0, N->stream>>>(N->d[1], N->e[0], N->c[0], N->n, 32, 16);
    conv(N, N->c[0], N->wb[6], B(6), N->d[0], 0, 48, 16, 1, false);
    conv(N, N->d[0], N->wb[7], B(7), N->y, 0, 16, 16, 0, true);
}

// Backward of one convolution: given dL/d(out) in gout (f32, [V][Cout]) and the
// layer's output (for the relu mask), accumulate dW, db, and write dL/d(in) (f32)
// into gin (overwrite).
void convBwd(vfem_net* N, int l, const bf16* in, const bf16* out, const float* gout, float* gin, bool wantIn) {
    const int lvl = kLevel[l], Cin = kCin[l], Cout = kCout[l];
    const int n = N->n >> lvl;
    const int64_t V = N->V[lvl];
    kReluMask<<<blocks(V * Cout), 256, 0, N->stream>>>(gout, out, N->gmask, V * Cout, kRelu[l]);
    kBiasGrad<<<Cout, 256, 0, N->stream>>>(N->gmask, N->gw + N->boff[l], V, Cout);
    const int chunks = (int)((V + WG_CHUNK - 1) / WG_CHUNK);
    dim3 gw((unsigned)chunks, 27, (unsigned)(((Cin + 63) / 64) * ((Cout + 63) / 64)));
    kConvWGrad<<<gw, 128, 0, N->stream>>>(in, N->gmask, N->wgPart, n, Cin, Cout);
    const int64_t per = 27LL * Cin * Cout;
    kWGradSum<<<blocks(per), 256, 0, N->stream>>>(N->wgPart, N->gw + N->woff[l], per, chunks);
    if (wantIn) conv(N, N->gmask, N->wt[l], nullptr, gin, lvl, Cout, Cin, 0, true);
}

void backward(vfem_net* N) {
    const int64_t* V = N->V;
    // y = conv7(d0)
    convBwd(N, 7, N->d[0], nullptr, N->gy, N->gd[0], true);
    // d0 = relu(conv6(c0))
    convBwd(N, 6, N->c[0], N->d[0], N->gd[0], N->gc[0], true);
    // c0 = [up(d1), e0]
    cudaMemsetAsync(N->ge[0], 0, sizeof(float) * V[0] * 16, N->stream);
    kUpConcatBwd<<<blocks(V[1] * 32 + V[0] * 16), 256, 0, N->stream>>>(N->gc[0], N->gd[1], N->ge[0], N->n, 32, 16);
    convBwd(N, 5, N->c[1], N->d[1], N->gd[1], N->gc[1], true);
    cudaMemsetAsync(N->ge[1], 0, sizeof(float) * V[1] * 32, N->stream);
    kUpConcatBwd<<<blocks(V[2] * 64 + V[1] * 32), 256, 0, N->stream>>>(N->gc[1], N->gd[2], N->ge[1], N->n / 2, 64, 32);
    convBwd(N, 4, N->c[2], N->d[2], N->gd[2], N->gc[2], true);
    cudaMemsetAsync(N->ge[2], 0, sizeof(float) * V[2] * 64, N->stream);
    kUpConcatBwd<<<blocks(V[3] * 128 + V[2] * 64), 256, 0, N->stream>>>(N->gc[2], N->ge[3], N->ge[2], N->n / 4, 128, 64);
    // e3 = relu(conv3(p3)); p3 = pool(e2)
    convBwd(N, 3, N->p[3], N->e[3], N->ge[3], N->gp[3], true);
    kPoolBwd<<<blocks(V[2] * 64), 256, 0, N->stream>>>(N->gp[3], N->ge[2], N->n / 8, 64, 1);
    convBwd(N, 2, N->p[2], N->e[2], N->ge[2], N->gp[2], true);
    kPoolBwd<<<blocks(V[1] * 32), 256, 0, N->stream>>>(N->gp[2], N->ge[1], N->n / 4, 32, 1);
    convBwd(N, 1, N->p[1], N->e[1], N->ge[1], N->gp[1], true);
    kPoolBwd<<<blocks(V[0] * 16), 256, 0, N->stream>>>(N->gp[1], N->ge[0], N->n / 2, 16, 1);
    convBwd(N, 0, N->x, N->e[0], N->ge[0], nullptr, false);
}

}  // namespace

extern "C" {

const char* vfem_net_last_error_message(void) { return g_netError.c_str(); }

vfem_status vfem_net_create(int32_t n, vfem_net** out) {
    if (!out || n < 8 || n % 8 != 0 || n > 512) return netFail(VFEM_ERR_INVALID_ARGUMENT, "grid size must be a multiple of 8 in [8, 512]");
    *out = nullptr;
    vfem_net* N = new vfem_net();
    N->n = n;
    for (int l = 0; l < 4; ++l) N->V[l] = (int64_t)(n >> l) * (n >> l) * (n >> l);
    int64_t off = 0;
    for (int l = 0; l < kLayers; ++l) {
        N->woff[l] = off;
        off += 27LL * kCin[l] * kCout[l];
        N->boff[l] = off;
        off += kCout[l];
    }
    N->nparam = off;
    auto bail = [&](cudaError_t e) {
        vfem_net_destroy(N);
        return netFail(VFEM_ERR_CUDA, std::string("allocation: ") + cudaGetErrorString(e));
    };
#define NA(call)                    \
    do {                            \
        cudaError_t e_ = (call);    \
        if (e_ != cudaSuccess) return bail(e_); \
    } while (0)
    NA(cudaStreamCreateWithFlags(&N->stream, cudaStreamNonBlocking));
    NA(nalloc(&N->w, off)); NA(nalloc(&N->gw, off)); NA(nalloc(&N->m, off)); NA(nalloc(&N->v, off));
    for (int l = 0; l < kLayers; ++l) {
        NA(nalloc(&N->wb[l], 27LL * kCin[l] * kCout[l]));
        NA(nalloc(&N->wt[l], 27LL * kCin[l] * kCout[l]));
    }
    const int64_t* V = N->V;
    NA(nalloc(&N->x, V[0] * 16));
    const int ec[4] = {16, 32, 64, 128};
    for (int l = 0; l < 4; ++l) {
        NA(nalloc(&N->e[l], V[l] * ec[l]));
        NA(nalloc(&N->ge[l], V[l] * ec[l]));
    }
    const int pc[4] = {0, 16, 32, 64};
    for (int l = 1; l < 4; ++l) {
        NA(nalloc(&N->p[l], V[l] * pc[l]));
        NA(nalloc(&N->gp[l], V[l] * pc[l]));
    }
    const int cc[3] = {48, 96, 192}, dc[3] = {16, 32, 64};
    for (int l = 0; l < 3; ++l) {
        NA(nalloc(&N->c[l], V[l] * cc[l]));
        NA(nalloc(&N->gc[l], V[l] * cc[l]));
        NA(nalloc(&N->d[l], V[l] * dc[l]));
        NA(nalloc(&N->gd[l], V[l] * dc[l]));
    }
    NA(nalloc(&N->y, V[0] * 16));
    NA(nalloc(&N->gy, V[0] * 16));
    NA(nalloc(&N->t, V[0] * 3));
    NA(nalloc(&N->mask, V[0]));
    int64_t gmax = 0;
    for (int l = 0; l < kLayers; ++l) gmax = std::max<int64_t>(gmax, V[kLevel[l]] * std::max(kCin[l], kCout[l]));
    NA(nalloc(&N->gmask, gmax));
    NA(nalloc(&N->gbf, gmax));
    int64_t wmax = 0;
    for (int l = 0; l < kLayers; ++l)
        wmax = std::max<int64_t>(wmax, (V[kLevel[l]] + WG_CHUNK - 1) / WG_CHUNK * 27 * kCin[l] * kCout[l]);
    NA(nalloc(&N->wgPart, wmax));
    NA(nalloc(&N->part, 4096));
    NA(cudaMallocHost((void**)&N->hostStage, sizeof(float) * V[0] * 16));
#undef NA
    *out = N;
    return VFEM_OK;
}

void vfem_net_destroy(vfem_net* N) {
    if (!N) return;
    cudaFree(N->w); cudaFree(N->gw); cudaFree(N->m); cudaFree(N->v);
    for (int l = 0; l < kLayers; ++l) { cudaFree(N->wb[l]); cudaFree(N->wt[l]); }
    cudaFree(N->x);
    for (int l = 0; l < 4; ++l) { cudaFree(N->e[l]); cudaFree(N->ge[l]); cudaFree(N->p[l]); cudaFree(N->gp[l]); }
    for (int l = 0; l < 3; ++l) { cudaFree(N->c[l]); cudaFree(N->gc[l]); cudaFree(N->d[l]); cudaFree(N->gd[l]); }
    cudaFree(N->y); cudaFree(N->gy); cudaFree(N->t); cudaFree(N->mask); cudaFree(N->gmask); cudaFree(N->gbf);
    cudaFree(N->part); cudaFree(N->wgPart);
    if (N->hostStage) cudaFreeHost(N->hostStage);
    if (N->stream) cudaStreamDestroy(N->stream);
    delete N;
}

int64_t vfem_net_num_params(const vfem_net* N) { return N ? N->nparam : 0; }

vfem_status vfem_net_set_params(vfem_net* N, const float* params) {
    if (!N || !params) return netFail(VFEM_ERR_INVALID_ARGUMENT, "null argument");
    NCK(cudaMemcpyAsync(N->w, params, sizeof(float) * N->nparam, cudaMemcpyHostToDevice, N->stream));
    NCK(cudaMemsetAsync(N->m, 0, sizeof(float) * N->nparam, N->stream));
    NCK(cudaMemsetAsync(N->v, 0, sizeof(float) * N->nparam, N->stream));
    N->step = 0;
    NCK(cudaStreamSynchronize(N->stream));
    return VFEM_OK;
}

vfem_status vfem_net_get_params(vfem_net* N, float* params) {
    if (!N || !params) return netFail(VFEM_ERR_INVALID_ARGUMENT, "null argument");
    NCK(cudaMemcpyAsync(params, N->w, sizeof(float) * N->nparam, cudaMemcpyDeviceToHost, N->stream));
    NCK(cudaStreamSynchronize(N->stream));
    return VFEM_OK;
}

// input: [n^3][16] FP32 features (channels beyond the used ones zero); output [n^3][3].
vfem_status vfem_net_forward(vfem_net* N, const float* input, float* output) {
    if (!N || !input || !output) return netFail(VFEM_ERR_INVALID_ARGUMENT, "null argument");
    const int64_t V = N->V[0];
    std::memcpy(N->hostStage, input, sizeof(float) * V * 16);
    NCK(cudaMemcpyAsync(N->gy, N->hostStage, sizeof(float) * V * 16, cudaMemcpyHostToDevice, N->stream));
    kF32ToBf16<<<blocks(V * 16), 256, 0, N->stream>>>(N->gy, N->x, V * 16);
    forward(N);
    NCK(cudaGetLastError());
    NCK(cudaMemcpyAsync(N->hostStage, N->y, sizeof(float) * V * 16, cudaMemcpyDeviceToHost, N->stream));
    NCK(cudaStreamSynchronize(N->stream));
    for (int64_t v = 0; v < V; ++v)
        for (int c = 0; c < 3; ++c) output[v * 3 + c] = N->hostStage[v * 16 + c];
    return VFEM_OK;
}

// Forward + backward of a batch of `batch` samples; gradients (summed over the
// batch, divided by it) to grads (host, nparam) if given, Adam step with lr if
// lr > 0.  loss_out: mean masked MSE.
vfem_status vfem_net_train_batch(vfem_net* N, const float* inputs, const float* targets, const float* masks,
                                 int32_t batch, float lr, float* grads, float* loss_out) {
    if (!N || !inputs || !targets || !masks || batch < 1) return netFail(VFEM_ERR_INVALID_ARGUMENT, "bad argument");
    const int64_t V = N->V[0];
    NCK(cudaMemsetAsync(N->gw, 0, sizeof(float) * N->nparam, N->stream));
    double lossSum = 0.0;
    std::vector<double> part(1024);
    for (int b = 0; b < batch; ++b) {
        std::memcpy(N->hostStage, inputs + (int64_t)b * V * 16, sizeof(float) * V * 16);
        NCK(cudaMemcpyAsync(N->gy, N->hostStage, sizeof(float) * V * 16, cudaMemcpyHostToDevice, N->stream));
        kF32ToBf16<<<blocks(V * 16), 256, 0, N->stream>>>(N->gy, N->x, V * 16);
        NCK(cudaMemcpyAsync(N->t, targets + (int64_t)b * V * 3, sizeof(float) * V * 3, cudaMemcpyHostToDevice, N->stream));
        NCK(cudaMemcpyAsync(N->mask, masks + (int64_t)b * V, sizeof(float) * V, cudaMemcpyHostToDevice, N->stream));
        forward(N);
        double cnt = 0.0;
        for (int64_t v = 0; v < V; ++v) cnt += masks[(int64_t)b * V + v];
        const float invCount = cnt > 0 ? (float)(1.0 / (3.0 * cnt)) : 0.f;
        kMse<<<1024, 256, 0, N->stream>>>(N->y, N->t, N->mask, N->gy, N->part, V, 16, invCount);
        backward(N);
        NCK(cudaMemcpyAsync(part.data(), N->part, sizeof(double) * 1024, cudaMemcpyDeviceToHost, N->stream));
        NCK(cudaStreamSynchronize(N->stream));
        double s = 0.0;
        for (double p : part) s += p;
        lossSum += s * invCount;
    }
    NCK(cudaGetLastError());
    if (loss_out) *loss_out = (float)(lossSum / batch);
    if (grads) {
        NCK(cudaMemcpyAsync(grads, N->gw, sizeof(float) * N->nparam, cudaMemcpyDeviceToHost, N->stream));
        NCK(cudaStreamSynchronize(N->stream));
        for (int64_t i = 0; i < N->nparam; ++i) grads[i] /= (float)batch;
    }
    if (lr > 0.f) {
        N->step++;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.f - std::pow(b1, (float)N->step), c2 = 1.f - std::pow(b2, (float)N->step);
        kAdam<<<blocks(N->nparam), 256, 0, N->stream>>>(N->w, N->gw, N->m, N->v, N->nparam, lr, b1, b2, 1e-8f, c1, c2,
                                                        1.f / (float)batch);
        NCK(cudaGetLastError());
        NCK(cudaStreamSynchronize(N->stream));
    }
    return VFEM_OK;
}

}  // extern "C"
