// kernels.cu -- sm_103a kernels of the voxel MG-PCG solve.
//
// Kernel map (reference shader / routine it replaces, paths relative to the
// reference project root):
//   kMatvecH, kMatvec  MatxVec.comp + FixedNodes.comp + VecDotVec.comp
//                    (MatrixFreeSparse.hpp:197-214): atomic-free element-by-element
//                    product on a 2.5-D tile (kMatvecH: Walsh-factorised isotropic
//                    cube Ke; kMatvec: general Ke), fixed rows zeroed, dots fused.
//   kRestrict2, kRestrict  CWiseMult.comp + Restrict.comp (MultigridPreconditioner.hpp:67-108):
//                    full weighting on the dense grid (kRestrict2<T, true> also
//                    performs the mixed solve's residual update, ConjugateGradient_1.comp).
//   kProlongFlat, kProlongSmooth2, kProlongSmooth  Interpolate.comp + PreSmoothAndAXPY.comp +
//                    Smooth.comp (MultigridPreconditioner.hpp:110-155,176-181),
//                    fixed mask and r.z fused.
//   kCoarseGather/kSymRuns/kSymRunsReduce, kGemv64  the coarsest SimplicialLDLT solve
//                    (MultigridPreconditioner.hpp:174-175) as a dense symmetric
//                    inverse: FP16 packed half tiles (mixed) or the full FP64 matrix.
//   kUpdateXR, kUpdateR  ConjugateGradient_1.comp + VecDotVec.comp (r.r).
//   kUpdateP, kUpdatePX  ConjugateGradient_2.comp (kUpdatePX: with the mixed solve's
//                    deferred x update).
// Reductions are deterministic: block partials in a fixed grid, summed in a
// fixed order by the last block to finish (no floating-point atomics).
#include <cfloat>
#include <cstdio>
#include <mutex>
#include <type_traits>

#include "kernels.h"
#include "reduce.cuh"

namespace vfem {

namespace {

constexpr int MV_TX = 32, MV_TY = 8, MV_ZC = 32;  // z layers per product block (32: 5% faster than 16)
constexpr int NT = 256;
constexpr int PZ = 8;  // z nodes per thread in the per-node kernels

// Double-float ("df") numbers: the unevaluated sum hi + lo of two FP32 values,
// about 48 significant bits, computed with FP32 instructions only (Dekker 1971:
// TwoSum / FastTwoSum; the product error from one FMA).  GB300 issues FP64 at
// about 1/64 of its FP32 rate, so the mixed-precision solve evaluates its true
// residual f - K x in df: relative rounding ~1e-14 of the summed magnitudes,
// several times faster than the FP64 product.  Addition is the "sloppy" variant
// (error bounded by ~2^-44 (|a| + |b|)), ample for a residual that is compared
// with 1e-6 |f|.  The compiler must not re-associate these expressions, which
// nvcc does not do without fast-math flags.
struct df {
    float hi, lo;
    df() = default;
    __host__ __device__ constexpr df(float h, float l) : hi(h), lo(l) {}
    __host__ __device__ constexpr explicit df(int v) : hi((float)v), lo(0.f) {}
    __host__ __device__ constexpr explicit df(float v) : hi(v), lo(0.f) {}
    __host__ __device__ explicit df(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
};

__device__ __forceinline__ df dfTwoSum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return df(s, (a - (s - bb)) + (b - bb));
}
__device__ __forceinline__ df dfFastTwoSum(float a, float b) {  // |a| >= |b|
    const float s = a + b;
    return df(s, b - (s - a));
}
__device__ __forceinline__ df operator+(df a, df b) {
    const df s = dfTwoSum(a.hi, b.hi);
    return dfFastTwoSum(s.hi, s.lo + (a.lo + b.lo));
}
__device__ __forceinline__ df operator-(df a, df b) { return a + df(-b.hi, -b.lo); }
__device__ __forceinline__ df operator*(df a, df b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return dfFastTwoSum(p, e);
}
__device__ __forceinline__ df& operator+=(df& a, df b) { return a = a + b; }
__device__ __forceinline__ df& operator*=(df& a, df b) { return a = a * b; }
// The df overload below would hide the global fma from unqualified calls in
// this namespace; these restore the FP32 and FP64 forms.
__device__ __forceinline__ float fma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fma(double a, double b, double c) { return ::fma(a, b, c); }
// a * b + c with one renormalisation.
__device__ __forceinline__ df fma(df a, df b, df c) {
    const float p = a.hi * b.hi;
    const float pe = fmaf(a.hi, b.hi, -p);
    const df s = dfTwoSum(p, c.hi);
    float t = s.lo + (pe + c.lo);
    t = fmaf(a.hi, b.lo, t);
    t = fmaf(a.lo, b.hi, t);
    return dfFastTwoSum(s.hi, t);
}

// Conversions between a storage type T and a compute type TC of the matvec.
template <typename T, typename TC>
struct Cvt {
    static __device__ __forceinline__ TC in(T v) { return TC(v); }
    static __device__ __forceinline__ T out(TC v) { return T(v); }
};
template <>
struct Cvt<double, df> {
    static __device__ __forceinline__ df in(double v) {
        const float h = __double2float_rn(v);
        return df(h, __double2float_rn(v - (double)h));
    }
    static __device__ __forceinline__ double out(df v) { return (double)v.hi + (double)v.lo; }
};
__device__ __forceinline__ float toF(float v) { return v; }
__device__ __forceinline__ float toF(double v) { return (float)v; }
__device__ __forceinline__ float toF(df v) { return v.hi; }  // hi is v rounded to FP32

template <>
struct DotAcc<df> {
    df s = df(0.f, 0.f);
    __device__ __forceinline__ void add(df v) { s = s + v; }
    __device__ __forceinline__ double get() const { return (double)s.hi + (double)s.lo; }
};

template <typename T>
struct Ks {
    T v[45];
};
template <typename T>
struct Kd {
    T v[576];
};

// y = Khat u on the 45-entry pattern (modes 1..7; mode 0, the rigid translation,
// has no energy).  u and y hold 3 m + c for mode m and component c.
template <typename T>
__device__ __forceinline__ void applyKhat(const T (&u)[24], T (&y)[24], const Ks<T>& k) {
#pragma unroll
    for (int i = 0; i < 24; ++i) y[i] = T(0);
#define KS_(n, r, c) y[r] = fma(k.v[n], u[c], y[r]);
    KS_(0, 3, 3) KS_(1, 3, 7) KS_(2, 3, 14) KS_(3, 7, 3) KS_(4, 7, 7) KS_(5, 7, 14) KS_(6, 14, 3) KS_(7, 14, 7)
    KS_(8, 14, 14)
    KS_(9, 6, 6) KS_(10, 6, 4) KS_(11, 4, 6) KS_(12, 4, 4) KS_(13, 23, 23)
    KS_(14, 12, 12) KS_(15, 12, 5) KS_(16, 5, 12) KS_(17, 5, 5) KS_(18, 22, 22)
    KS_(19, 13, 13) KS_(20, 13, 8) KS_(21, 8, 13) KS_(22, 8, 8) KS_(23, 21, 21)
    KS_(24, 10, 10) KS_(25, 10, 17) KS_(26, 17, 10) KS_(27, 17, 17)
    KS_(28, 9, 9) KS_(29, 9, 20) KS_(30, 20, 9) KS_(31, 20, 20)
    KS_(32, 15, 15) KS_(33, 15, 19) KS_(34, 19, 15) KS_(35, 19, 19)
    KS_(36, 18, 18) KS_(37, 18, 16) KS_(38, 18, 11) KS_(39, 16, 18) KS_(40, 16, 16) KS_(41, 16, 11)
    KS_(42, 11, 18) KS_(43, 11, 16) KS_(44, 11, 11)
#undef KS_
}

// y = e * Ke u, general symmetric Ke.
template <typename T>
__device__ __forceinline__ void elemDense(const T (&u)[24], T (&y)[24], const Kd<T>& k, T e) {
#pragma unroll
    for (int r = 0; r < 24; ++r) {
        T s = T(0);
#pragma unroll
        for (int c = 0; c < 24; ++c) s = fma(k.v[r * 24 + c], u[c], s);
        y[r] = s * e;
    }
}

// Shared-memory node slots are padded to 4 values (x, y, z, unused) so that a
// node moves with one 16-byte (float) or two 16-byte (double) accesses.
constexpr int kSuElems = 2 * (MV_TY + 1) * (MV_TX + 1) * 4;
constexpr int kSyElems = MV_TY * MV_TX * 6 * 4;

template <typename T>
__device__ __forceinline__ void stSlot(T* p, T a, T b, T c);
template <>
__device__ __forceinline__ void stSlot<float>(float* p, float a, float b, float c) {
    *reinterpret_cast<float4*>(p) = make_float4(a, b, c, 0.f);
}
template <>
__device__ __forceinline__ void stSlot<double>(double* p, double a, double b, double c) {
    reinterpret_cast<double2*>(p)[0] = make_double2(a, b);
    reinterpret_cast<double2*>(p)[1] = make_double2(c, 0.0);
}
template <>
__device__ __forceinline__ void stSlot<df>(df* p, df a, df b, df c) {
    reinterpret_cast<float4*>(p)[0] = make_float4(a.hi, a.lo, b.hi, b.lo);
    reinterpret_cast<float4*>(p)[1] = make_float4(c.hi, c.lo, 0.f, 0.f);
}
template <typename T>
__device__ __forceinline__ void ldSlot(const T* p, T& a, T& b, T& c);
template <>
__device__ __forceinline__ void ldSlot<df>(const df* p, df& a, df& b, df& c) {
    const float4 v0 = reinterpret_cast<const float4*>(p)[0], v1 = reinterpret_cast<const float4*>(p)[1];
    a = df(v0.x, v0.y);
    b = df(v0.z, v0.w);
    c = df(v1.x, v1.y);
}
template <>
__device__ __forceinline__ void ldSlot<float>(const float* p, float& a, float& b, float& c) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    a = v.x;
    b = v.y;
    c = v.z;
}
template <>
__device__ __forceinline__ void ldSlot<double>(const double* p, double& a, double& b, double& c) {
    const double2 v0 = reinterpret_cast<const double2*>(p)[0], v1 = reinterpret_cast<const double2*>(p)[1];
    a = v0.x;
    b = v0.y;
    c = v1.x;
}

// Output stage of the matvec kernels for one owned node s: sum = (K x)_s before
// the fixed-row mask; writes y (and y32) by mode and accumulates the dots.  fl:
// the node's flags.  The x.(Kx) term skips unused and fixed nodes, where Kx is
// 0, so that whatever x holds there (the caller's buffer may carry NaN at nodes
// no element touches) cannot reach the dot.
template <typename T, typename TC>
__device__ __forceinline__ void mvOutput(const MatvecArgs<T>& a, int64_t s, const TC (&sum)[3], uint8_t fl,
                                         const TC (&xo)[3], DotAcc<TC>& d0, DotAcc<TC>& d1) {
    typedef Cvt<T, TC> C;
    const bool fixed = (fl & FLAG_FIXED) != 0;
    const bool live = (fl & FLAG_USED) && !fixed;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const TC ax = fixed ? TC(0) : sum[c];
        TC out;
        TC fv = TC(0);
        if (a.mode != MV_AX) fv = C::in(a.f[3 * s + c]);
        const TC xv = xo[c];
        switch (a.mode) {
            case MV_AX: out = ax; break;
            case MV_RESID: out = fv - ax; break;
            case MV_RESID0: out = fixed ? TC(0) : fv - ax; break;
            default: out = fixed ? TC(0) : xv + TC(a.omega) * C::in(a.dinv[3 * s + c]) * (fv - ax); break;
        }
        if constexpr (std::is_same<T, TC>::value) a.y[3 * s + c] = out;
        else if (a.y) a.y[3 * s + c] = C::out(out);
        if (a.y32) a.y32[3 * s + c] = toF(out);
        if (a.dot0 == DOT_X_OUT) d0.add(live ? xv * out : TC(0));
        else if (a.dot0 == DOT_OUT_OUT) d0.add(out * out);
        else if (a.dot0 == DOT_F_OUT) d0.add(fv * out);
        if (a.dot1) d1.add(out * C::in(a.aux[3 * s + c]));
    }
}

// Element-by-element product with a general (dense 24 x 24) Ke, for element
// matrices without the isotropic-cube symmetry (for example the reference's
// Ke0.dat in its own node order); structured Ke use kMatvecH below.
// A 2.5-D tile: a block of 32 x 8 threads marches
// up a z-range; at each element layer thread (tx,ty) computes the element whose
// lower corner is node (x0+tx-1, y0+ty-1) and owns node (x0+tx, y0+ty), which is
// the (1,1) corner of its own element and a corner of the three neighbouring
// threads' elements.  Element outputs pass through shared memory once; each
// owned node sums its four in-layer contributions for the bottom face (node
// layer k) and the top face (node layer k+1), so no atomics are needed.
// The march is software-pipelined: while layer k is computed, the node values
// of layer k+2, the modulus of element layer k+1 and the owned node's flags
// are already in flight to registers.  The 33 x 9 node tile of a layer is
// loaded without integer division: every thread loads its own slot, row 8
// comes from the ty == 0 threads and column 32 from nine threads of row 1.
//
// T is the storage type of the vectors, TC the arithmetic type (T, or df for
// the true residual of the mixed-precision solve: FP64 vectors, df arithmetic).
template <typename T, typename TC = T>
__global__ void __launch_bounds__(MV_TX* MV_TY, 1)
    kMatvec(MatvecArgs<T> a, const Kd<TC> kp, Scalars* S, RedBuf rb) {
    if (a.checkDone && S->done) return;
    if (a.condTrue && !trueResidualDue(S)) return;
    typedef Cvt<T, TC> C;
    extern __shared__ __align__(16) unsigned char smemRaw[];
    TC* su = reinterpret_cast<TC*>(smemRaw);
    TC* sy = su + kSuElems;
    const Grid g = a.g;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x0 = blockIdx.x * (MV_TX - 1), y0 = blockIdx.y * (MV_TY - 1), z0 = blockIdx.z * MV_ZC;
    const int zend = min(z0 + MV_ZC, g.nz);
    const int64_t plane = (int64_t)g.nx * g.ny;
    const int ecx = x0 + tx - 1, ecy = y0 + ty - 1;
    const int onx = x0 + tx, ony = y0 + ty;
    const bool owner = (tx < MV_TX - 1) && (ty < MV_TY - 1) && onx < g.nx && ony < g.ny;
    const bool ecxy = ecx >= 0 && ecx < g.ex && ecy >= 0 && ecy < g.ey;
    const int eCol = ecy * g.nx + ecx;   // in-plane offsets fit in 32 bits for every accepted grid
    const int oCol = ony * g.nx + onx;
    const TC sc = TC(a.scale);
    // Extra tile slots: row MV_TY (ty == 0 threads), column MV_TX (row-1 threads tx <= MV_TY).
    const bool hasR = ty == 0, hasC = (ty == 1) && (tx <= MV_TY);
    const int rX = x0 - 1 + tx, rY = y0 - 1 + MV_TY;
    const int cX = x0 - 1 + MV_TX, cY = y0 - 1 + tx;
    const bool ok0 = ecx >= 0 && ecx < g.nx && ecy >= 0 && ecy < g.ny;
    const bool okR = hasR && rX >= 0 && rX < g.nx && rY >= 0 && rY < g.ny;
    const bool okC = hasC && cX >= 0 && cX < g.nx && cY >= 0 && cY < g.ny;
#define SU(b, iy, ix) (su + (((((b) * (MV_TY + 1)) + (iy)) * (MV_TX + 1) + (ix)) << 2))
#define SY(k, iy, ix) (sy + (((((k) * MV_TY) + (iy)) * MV_TX + (ix)) << 2))
    T pf[9];
    auto gload = [&](int zl) {
        const bool zok = zl >= 0 && zl < g.nz;
        const int64_t zoff = (int64_t)zl * plane;
#pragma unroll
        for (int i = 0; i < 9; ++i) pf[i] = T(0);
        if (ok0 && zok) {
            const T* p = a.x + 3 * ((int64_t)eCol + zoff);
            pf[0] = p[0]; pf[1] = p[1]; pf[2] = p[2];
        }
        if (okR && zok) {
            const T* p = a.x + 3 * ((int64_t)(rY * g.nx + rX) + zoff);
            pf[3] = p[0]; pf[4] = p[1]; pf[5] = p[2];
        }
        if (okC && zok) {
            const T* p = a.x + 3 * ((int64_t)(cY * g.nx + cX) + zoff);
            pf[6] = p[0]; pf[7] = p[1]; pf[8] = p[2];
        }
    };
    auto sstore = [&](int zl) {
        const int b = zl & 1;
        stSlot<TC>(SU(b, ty, tx), C::in(pf[0]), C::in(pf[1]), C::in(pf[2]));
        if (hasR) stSlot<TC>(SU(b, MV_TY, tx), C::in(pf[3]), C::in(pf[4]), C::in(pf[5]));
        if (hasC) stSlot<TC>(SU(b, tx, MV_TX), C::in(pf[6]), C::in(pf[7]), C::in(pf[8]));
    };
    auto eload = [&](int k) -> float {
        return (ecxy && k >= 0 && k < g.ez) ? a.E[(int64_t)eCol + (int64_t)k * plane] : 0.f;
    };
    auto fload = [&](int k) -> uint8_t {
        return (owner && k >= z0 && k < zend) ? a.flags[(int64_t)oCol + (int64_t)k * plane] : (uint8_t)0;
    };
    TC acc[3] = {TC(0), TC(0), TC(0)};
    DotAcc<TC> d0, d1;
    gload(z0 - 1);
    sstore(z0 - 1);
    gload(z0);
    float Enext = eload(z0 - 1);
    uint8_t flNext = fload(z0 - 1);
    for (int k = z0 - 1; k < zend; ++k) {
        sstore(k + 1);
        const float Ee = Enext;
        const uint8_t fl = flNext;
        __syncthreads();
        gload(k + 2);           // consumed by the next iteration
        Enext = eload(k + 1);
        flNext = fload(k + 1);
        // x at the owned node of layer k, read now: the next iteration's store
        // overwrites this layer's buffer without waiting for the output phase.
        TC xo[3];
        ldSlot<TC>(SU(k & 1, ty + 1, tx + 1), xo[0], xo[1], xo[2]);
        TC ye[24];
        if (Ee != 0.f) {
            TC u[24];
#pragma unroll
            for (int n = 0; n < 8; ++n) {
                const int dx = n & 1, dy = (n >> 1) & 1, dz = n >> 2;
                ldSlot<TC>(SU((k + dz) & 1, ty + dy, tx + dx), u[3 * n], u[3 * n + 1], u[3 * n + 2]);
            }
            elemDense<TC>(u, ye, kp, sc * TC(Ee));
        } else {
#pragma unroll
            for (int i = 0; i < 24; ++i) ye[i] = TC(0);
        }
        stSlot<TC>(SY(0, ty, tx), ye[0], ye[1], ye[2]);     // a = 0
        stSlot<TC>(SY(1, ty, tx), ye[3], ye[4], ye[5]);     // a = 1
        stSlot<TC>(SY(2, ty, tx), ye[6], ye[7], ye[8]);     // a = 2
        stSlot<TC>(SY(3, ty, tx), ye[12], ye[13], ye[14]);  // a = 4
        stSlot<TC>(SY(4, ty, tx), ye[15], ye[16], ye[17]);  // a = 5
        stSlot<TC>(SY(5, ty, tx), ye[18], ye[19], ye[20]);  // a = 6
        __syncthreads();
        if (owner) {
            TC lo[3], hi[3], q[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                lo[c] = ye[9 + c];
                hi[c] = ye[21 + c];
            }
            ldSlot<TC>(SY(2, ty, tx + 1), q[0], q[1], q[2]);
#pragma unroll
            for (int c = 0; c < 3; ++c) lo[c] += q[c];
            ldSlot<TC>(SY(1, ty + 1, tx), q[0], q[1], q[2]);
#pragma unroll
            for (int c = 0; c < 3; ++c) lo[c] += q[c];
            ldSlot<TC>(SY(0, ty + 1, tx + 1), q[0], q[1], q[2]);
#pragma unroll
            for (int c = 0; c < 3; ++c) lo[c] += q[c];
            ldSlot<TC>(SY(5, ty, tx + 1), q[0], q[1], q[2]);
#pragma unroll
            for (int c = 0; c < 3; ++c) hi[c] += q[c];
            ldSlot<TC>(SY(4, ty + 1, tx), q[0], q[1], q[2]);
#pragma unroll
            for (int c = 0; c < 3; ++c) hi[c] += q[c];
            ldSlot<TC>(SY(3, ty + 1, tx + 1), q[0], q[1], q[2]);
#pragma unroll
            for (int c = 0; c < 3; ++c) hi[c] += q[c];
            if (k >= z0) {
                TC sum[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) sum[c] = acc[c] + lo[c];
                mvOutput<T, TC>(a, (int64_t)oCol + (int64_t)k * plane, sum, fl, xo, d0, d1);
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) acc[c] = hi[c];
        }
    }
#undef SU
#undef SY
    if (a.epi != EPI_NONE) {
        double v[2] = {d0.get(), d1.get()}, t[2];
        if (gridReduce<MV_TX * MV_TY, 2>(v, rb, t)) applyEpi(a.epi, S, t[0], t[1]);
    }
}

// 4-point Walsh-Hadamard transform of a node quad (corner q = dx + 2 dy), per
// component: v[3m+c] = sum_q (-1)^popcount(m&q) u[3q+c].
template <typename T>
__device__ __forceinline__ void fwht4x3(T (&v)[12]) {
#pragma unroll
    for (int s = 1; s < 4; s <<= 1) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (q & s) continue;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const T p = v[3 * q + c], r = v[3 * (q + s) + c];
                v[3 * q + c] = p + r;
                v[3 * (q + s) + c] = p - r;
            }
        }
    }
}

// FP32: the x and y components of a node move as one register pair through
// the packed FP32x2 instructions (same IEEE results; p - r as fma(r, -1, p) is
// exact before its rounding), the z component alone: 2/3 of the instructions.
__device__ __forceinline__ float2 pr2(const float* v) { return make_float2(v[0], v[1]); }
__device__ __forceinline__ void st2(float* v, float2 a) {
    v[0] = a.x;
    v[1] = a.y;
}
__device__ __forceinline__ float2 sub2(float2 p, float2 r) { return __ffma2_rn(r, make_float2(-1.f, -1.f), p); }
__device__ __forceinline__ void bfly3(float* a, float* b) {
    const float2 p = pr2(a), r = pr2(b);
    st2(a, __fadd2_rn(p, r));
    st2(b, sub2(p, r));
    const float pz = a[2], rz = b[2];
    a[2] = pz + rz;
    b[2] = pz - rz;
}
template <>
__device__ __forceinline__ void fwht4x3<float>(float (&v)[12]) {
    bfly3(v, v + 3);
    bfly3(v + 6, v + 9);
    bfly3(v, v + 6);
    bfly3(v + 3, v + 9);
}

// uh = (qb + qt, qb - qt) (24 values).
template <typename T>
__device__ __forceinline__ void sumDiff12(const T (&a)[12], const T (&b)[12], T (&u)[24]) {
#pragma unroll
    for (int i = 0; i < 12; ++i) {
        u[i] = a[i] + b[i];
        u[12 + i] = a[i] - b[i];
    }
}
template <>
__device__ __forceinline__ void sumDiff12<float>(const float (&a)[12], const float (&b)[12], float (&u)[24]) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const float2 p = pr2(a + 3 * q), r = pr2(b + 3 * q);
        st2(u + 3 * q, __fadd2_rn(p, r));
        st2(u + 12 + 3 * q, sub2(p, r));
        u[3 * q + 2] = a[3 * q + 2] + b[3 * q + 2];
        u[12 + 3 * q + 2] = a[3 * q + 2] - b[3 * q + 2];
    }
}
// u[i] *= e for the modes 1..7 (i >= 3).
template <typename T>
__device__ __forceinline__ void scaleModes(T (&u)[24], T e) {
#pragma unroll
    for (int i = 3; i < 24; ++i) u[i] *= e;
}
template <>
__device__ __forceinline__ void scaleModes<float>(float (&u)[24], float e) {
#pragma unroll
    for (int m = 1; m < 8; ++m) {
        st2(u + 3 * m, __fmul2_rn(pr2(u + 3 * m), make_float2(e, e)));
        u[3 * m + 2] *= e;
    }
}
// nb = carry + (y_bottom + y_top); carry = y_bottom - y_top.
template <typename T>
__device__ __forceinline__ void foldCarry(const T (&y)[24], T (&carry)[12], T (&nb)[12]) {
#pragma unroll
    for (int i = 0; i < 12; ++i) {
        nb[i] = carry[i] + (y[i] + y[12 + i]);
        carry[i] = y[i] - y[12 + i];
    }
}
template <>
__device__ __forceinline__ void foldCarry<float>(const float (&y)[24], float (&carry)[12], float (&nb)[12]) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const float2 yb = pr2(y + 3 * q), yt = pr2(y + 12 + 3 * q), cr = pr2(carry + 3 * q);
        st2(nb + 3 * q, __fadd2_rn(cr, __fadd2_rn(yb, yt)));
        st2(carry + 3 * q, sub2(yb, yt));
        const float zb = y[3 * q + 2], zt = y[12 + 3 * q + 2];
        nb[3 * q + 2] = carry[3 * q + 2] + (zb + zt);
        carry[3 * q + 2] = zb - zt;
    }
}

// The structured (isotropic cube) product with the Walsh-Hadamard factors
// shared along z.  With corner a = (q, dz) and mode m = (mq, mz), the 8-point
// transform splits into the 4-point transforms Q_0, Q_1 of the element's bottom
// and top node quads: uh[(mq,0)] = Q_0 + Q_1, uh[(mq,1)] = Q_0 - Q_1.  The top
// quad's transform of element layer k is the bottom one of layer k+1, so each
// quad is transformed once.  On the way back the top-face output of layer k-1
// and the bottom-face output of layer k land on the same node quad and are
// added in the Walsh domain before one inverse 4-point transform.  Per element
// this halves the shared-memory node reads (4 instead of 8), the exported
// contributions (3 instead of 6) and the quad transforms, against kMatvec.
// Same tile, pipelining and output stage as kMatvec.  The two Walsh-domain
// carries stay in registers across the z march.  Launch bounds, measured on
// the 256^3 workload: FP32 3 blocks per SM (80 registers, no spills; 4 blocks
// spill and run 33% slower); FP64 and df 2 blocks per SM (128 registers, a few
// spilled values; 20% faster than 1 block without spills).
//
// OUT selects the output stage at compile time (runtime mode switches in the
// owner stage cost ~20% of this issue-bound kernel):
//   OUT_ANY   mvOutput with the runtime mode and dots;
//   OUT_CG    the CG product: y = Kx (fixed rows 0), dot x.(Kx); the per-thread
//             dot sums at most 48 terms and accumulates with plain FMAs;
//   OUT_TRUE  the true residual: r = f - Kx, its FP32 rounding to y32, y (FP64)
//             only when given, dot r.r;
//   OUT_CG_PX the CG product with the mixed solve's direction update fused into
//             the input stage: every staged node value is p = z + beta p_old
//             (halo copies computed the same way by every block that stages
//             them), and the thread that stages an owned node writes the new p
//             to the other p buffer and adds the deferred alpha p_old to the
//             FP32 solution correction.  The p buffers alternate (Scalars::pSel,
//             flipped by the last block), because neighbouring blocks still read
//             p_old as their halo.
enum MvOut : int { OUT_ANY = 0, OUT_CG = 1, OUT_TRUE = 2, OUT_CG_PX = 3 };
template <typename T, typename TC, int OUT = OUT_ANY>
__global__ void __launch_bounds__(MV_TX* MV_TY, sizeof(TC) == 4 ? 3 : 2)
    kMatvecH(MatvecArgs<T> a, const Ks<TC> kp, Scalars* S, RedBuf rb) {
    if (a.checkDone && S->done) return;
    if (a.condTrue && !trueResidualDue(S)) return;
    typedef Cvt<T, TC> C;
    extern __shared__ __align__(16) unsigned char smemRaw[];
    TC* su = reinterpret_cast<TC*>(smemRaw);
    TC* sy = su + kSuElems;
    const Grid g = a.g;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x0 = blockIdx.x * (MV_TX - 1), y0 = blockIdx.y * (MV_TY - 1), z0 = blockIdx.z * MV_ZC;
    const int zend = min(z0 + MV_ZC, g.nz);
    const int64_t plane = (int64_t)g.nx * g.ny;
    const int ecx = x0 + tx - 1, ecy = y0 + ty - 1;
    const int onx = x0 + tx, ony = y0 + ty;
    const bool owner = (tx < MV_TX - 1) && (ty < MV_TY - 1) && onx < g.nx && ony < g.ny;
    const bool ecxy = ecx >= 0 && ecx < g.ex && ecy >= 0 && ecy < g.ey;
    const int eCol = ecy * g.nx + ecx;
    const int oCol = ony * g.nx + onx;
    const TC sc = TC(a.scale);
    const bool hasR = ty == 0, hasC = (ty == 1) && (tx <= MV_TY);
    const int rX = x0 - 1 + tx, rY = y0 - 1 + MV_TY;
    const int cX = x0 - 1 + MV_TX, cY = y0 - 1 + tx;
    const bool ok0 = ecx >= 0 && ecx < g.nx && ecy >= 0 && ecy < g.ny;
    const bool okR = hasR && rX >= 0 && rX < g.nx && rY >= 0 && rY < g.ny;
    const bool okC = hasC && cX >= 0 && cX < g.nx && cY >= 0 && cY < g.ny;
#define SU(b, iy, ix) (su + (((((b) * (MV_TY + 1)) + (iy)) * (MV_TX + 1) + (ix)) << 2))
#define SY(k, iy, ix) (sy + (((((k) * MV_TY) + (iy)) * MV_TX + (ix)) << 2))
    // Input source; OUT_CG_PX: p_old, the buffer for the new p, beta and the
    // deferred alpha (0 when a flush has folded it).  Every block reads the
    // scalars here, before it reaches the grid reduction after which the last
    // block flips pSel and advances matvecs.
    const T* src = a.x;
    T* pNew = nullptr;
    T beta = T(0), ax = T(0);
    int sel = 0;
    if constexpr (OUT == OUT_CG_PX) {
        sel = S->pSel;
        src = sel ? a.pAlt : a.x;
        pNew = sel ? const_cast<T*>(a.x) : a.pAlt;
        beta = T(S->beta);
        ax = S->foldStamp == S->matvecs ? T(0) : T(S->alpha);
        if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && tx == 0 && ty == 0)
            S->pxStamp = S->matvecs;  // read only by kFlushX
    }
    // The thread that stages node (ecx, ecy) is the one after its owner in x and y.
    // OUT_CG_PX keeps the raw z, p_old (and, for an owned node, x) values of the
    // prefetched layer in registers and forms p = z + beta p_old when the layer
    // is staged to shared memory, so the prefetch stays in flight across the
    // element computation as in the plain product.
    const bool stagesOwned = OUT == OUT_CG_PX && tx >= 1 && ty >= 1;
    T pf[9];
    [[maybe_unused]] T pq[OUT == OUT_CG_PX ? 9 : 1], xq[OUT == OUT_CG_PX ? 3 : 1];
    auto ld3 = [&](int64_t i, int o) {
        pf[o] = src[i];
        pf[o + 1] = src[i + 1];
        pf[o + 2] = src[i + 2];
        if constexpr (OUT == OUT_CG_PX) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                pq[o + c] = pf[o + c];
                pf[o + c] = a.zin[i + c];
            }
        }
    };
    auto ownsLayer = [&](int zl) { return stagesOwned && ok0 && zl >= z0 && zl < zend; };
    auto gload = [&](int zl) {
        const bool zok = zl >= 0 && zl < g.nz;
        const int64_t zoff = (int64_t)zl * plane;
#pragma unroll
        for (int i = 0; i < 9; ++i) pf[i] = T(0);
        if constexpr (OUT == OUT_CG_PX) {
#pragma unroll
            for (int i = 0; i < 9; ++i) pq[i] = T(0);
        }
        if (ok0 && zok) {
            ld3(3 * ((int64_t)eCol + zoff), 0);
            if constexpr (OUT == OUT_CG_PX) {
                if (ax != T(0) && ownsLayer(zl)) {
                    const int64_t i = 3 * ((int64_t)eCol + zoff);
                    xq[0] = a.xacc[i];
                    xq[1] = a.xacc[i + 1];
                    xq[2] = a.xacc[i + 2];
                }
            }
        }
        if (okR && zok) ld3(3 * ((int64_t)(rY * g.nx + rX) + zoff), 3);
        if (okC && zok) ld3(3 * ((int64_t)(cY * g.nx + cX) + zoff), 6);
    };
    auto sstore = [&](int zl) {
        const int b = zl & 1;
        if constexpr (OUT == OUT_CG_PX) {
            if (beta != T(0)) {
#pragma unroll
                for (int i = 0; i < 9; ++i) pf[i] = fma(beta, pq[i], pf[i]);
            }
            if (ownsLayer(zl)) {
                const int64_t i = 3 * ((int64_t)eCol + (int64_t)zl * plane);
#pragma unroll
                for (int c = 0; c < 3; ++c) pNew[i + c] = pf[c];
                if (ax != T(0)) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) a.xacc[i + c] = fma(ax, pq[c], xq[c]);
                }
            }
        }
        stSlot<TC>(SU(b, ty, tx), C::in(pf[0]), C::in(pf[1]), C::in(pf[2]));
        if (hasR) stSlot<TC>(SU(b, MV_TY, tx), C::in(pf[3]), C::in(pf[4]), C::in(pf[5]));
        if (hasC) stSlot<TC>(SU(b, tx, MV_TX), C::in(pf[6]), C::in(pf[7]), C::in(pf[8]));
    };
    auto eload = [&](int k) -> float {
        return (ecxy && k >= 0 && k < g.ez) ? a.E[(int64_t)eCol + (int64_t)k * plane] : 0.f;
    };
    auto fload = [&](int k) -> uint8_t {
        return (owner && k >= z0 && k < zend) ? a.flags[(int64_t)oCol + (int64_t)k * plane] : (uint8_t)0;
    };
    // Walsh-domain quad of the current bottom node layer, and the top-face
    // output of the previous element layer (Walsh domain).
    TC qb[12], carry[12];
#pragma unroll
    for (int i = 0; i < 12; ++i) carry[i] = TC(0);
    DotAcc<TC> d0, d1;
    TC dAx = TC(0);  // OUT_CG: x.(Kx) of this thread
    gload(z0 - 1);
    sstore(z0 - 1);
    gload(z0);
    float Enext = eload(z0 - 1);
    uint8_t flNext = fload(z0 - 1);
    for (int k = z0 - 1; k < zend; ++k) {
        sstore(k + 1);
        const float Ee = Enext;
        const uint8_t fl = flNext;
        __syncthreads();
        gload(k + 2);
        Enext = eload(k + 1);
        flNext = fload(k + 1);
        TC xo[3];
        ldSlot<TC>(SU(k & 1, ty + 1, tx + 1), xo[0], xo[1], xo[2]);
        if (k == z0 - 1) {
#pragma unroll
            for (int q = 0; q < 4; ++q)
                ldSlot<TC>(SU(k & 1, ty + (q >> 1), tx + (q & 1)), qb[3 * q], qb[3 * q + 1], qb[3 * q + 2]);
            fwht4x3<TC>(qb);
        }
        TC qt[12];
#pragma unroll
        for (int q = 0; q < 4; ++q)
            ldSlot<TC>(SU((k + 1) & 1, ty + (q >> 1), tx + (q & 1)), qt[3 * q], qt[3 * q + 1], qt[3 * q + 2]);
        fwht4x3<TC>(qt);
        TC nb[12];  // node layer k: Walsh-domain contributions at the element's bottom quad
        if (Ee != 0.f) {
            TC uh[24], yh[24];
            const TC e = sc * TC(Ee);
            sumDiff12<TC>(qb, qt, uh);
            scaleModes<TC>(uh, e);
            applyKhat<TC>(uh, yh, kp);
            foldCarry<TC>(yh, carry, nb);
        } else {
#pragma unroll
            for (int i = 0; i < 12; ++i) {
                nb[i] = carry[i];
                carry[i] = TC(0);
            }
        }
#pragma unroll
        for (int i = 0; i < 12; ++i) qb[i] = qt[i];
        fwht4x3<TC>(nb);
        stSlot<TC>(SY(0, ty, tx), nb[0], nb[1], nb[2]);  // corner (0,0)
        stSlot<TC>(SY(1, ty, tx), nb[3], nb[4], nb[5]);  // corner (1,0)
        stSlot<TC>(SY(2, ty, tx), nb[6], nb[7], nb[8]);  // corner (0,1)
        __syncthreads();
        if (owner && k >= z0) {
            TC sum[3] = {nb[9], nb[10], nb[11]}, q[3];  // own corner (1,1)
            ldSlot<TC>(SY(2, ty, tx + 1), q[0], q[1], q[2]);
#pragma unroll
            for (int c = 0; c < 3; ++c) sum[c] += q[c];
            ldSlot<TC>(SY(1, ty + 1, tx), q[0], q[1], q[2]);
#pragma unroll
            for (int c = 0; c < 3; ++c) sum[c] += q[c];
            ldSlot<TC>(SY(0, ty + 1, tx + 1), q[0], q[1], q[2]);
#pragma unroll
            for (int c = 0; c < 3; ++c) sum[c] += q[c];
            const int64_t s = (int64_t)oCol + (int64_t)k * plane;
            if constexpr (OUT == OUT_CG || OUT == OUT_CG_PX) {
                const bool fixed = (fl & FLAG_FIXED) != 0;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const TC out = fixed ? TC(0) : sum[c];
                    a.y[3 * s + c] = C::out(out);
                    dAx = fma(xo[c], out, dAx);
                }
            } else if constexpr (OUT == OUT_TRUE) {
                const bool fixed = (fl & FLAG_FIXED) != 0;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const TC out = C::in(a.f[3 * s + c]) - (fixed ? TC(0) : sum[c]);
                    if (a.y) a.y[3 * s + c] = C::out(out);
                    a.y32[3 * s + c] = toF(out);
                    d0.add(out * out);
                }
            } else {
                mvOutput<T, TC>(a, s, sum, fl, xo, d0, d1);
            }
        }
    }
#undef SU
#undef SY
    if constexpr (OUT == OUT_CG || OUT == OUT_CG_PX) d0.add(dAx);
    if (a.epi != EPI_NONE) {
        double v[2] = {d0.get(), d1.get()}, t[2];
        if (gridReduce<MV_TX * MV_TY, 2>(v, rb, t)) {
            applyEpi(a.epi, S, t[0], t[1]);
            if constexpr (OUT == OUT_CG_PX) S->pSel = sel ^ 1;
        }
    }
}

// Full weighting (the transpose of trilinear prolongation) on the dense grid:
// rc[C] = sum_{|d| < DIV} prod_i (DIV - |d_i|)/DIV * rf[DIV*C + d].  Equal to
// the reference's W-weighted per-element restriction (see setup.cpp).
template <typename T, int DIV>
__global__ void __launch_bounds__(256) kRestrict(Grid gf, Grid gc, const T* __restrict__ rf, T* __restrict__ rc,
                                                 const Scalars* S, int checkDone) {
    if (checkDone && S->done) return;
    const int cx = blockIdx.x * 32 + threadIdx.x, cy = blockIdx.y * 8 + threadIdx.y;
    if (cx >= gc.nx || cy >= gc.ny) return;
    constexpr int R = DIV - 1;
    const T inv = T(1) / T(DIV);
    for (int cz = blockIdx.z * PZ; cz < min(gc.nz, (int)(blockIdx.z + 1) * PZ); ++cz) {
        T a0 = T(0), a1 = T(0), a2 = T(0);
        for (int dz = -R; dz <= R; ++dz) {
            const int fz = cz * DIV + dz;
            if (fz < 0 || fz >= gf.nz) continue;
            const T wz = T(DIV - abs(dz)) * inv;
            for (int dy = -R; dy <= R; ++dy) {
                const int fy = cy * DIV + dy;
                if (fy < 0 || fy >= gf.ny) continue;
                const T wy = T(DIV - abs(dy)) * inv;
                T s0 = T(0), s1 = T(0), s2 = T(0);
#pragma unroll
                for (int dx = -R; dx <= R; ++dx) {
                    const int fx = cx * DIV + dx;
                    if (fx < 0 || fx >= gf.nx) continue;
                    const T wx = T(DIV - abs(dx)) * inv;
                    const T* p = rf + 3 * gf.store(fx, fy, fz);
                    s0 = fma(wx, p[0], s0);
                    s1 = fma(wx, p[1], s1);
                    s2 = fma(wx, p[2], s2);
                }
                const T w = wz * wy;
                a0 = fma(w, s0, a0);
                a1 = fma(w, s1, a1);
                a2 = fma(w, s2, a2);
            }
        }
        T* q = rc + 3 * gc.store(cx, cy, cz);
        q[0] = a0;
        q[1] = a1;
        q[2] = a2;
    }
}

// Trilinear prolongation of coarse node values to fine node (fx,fy,fz).
// The same full weighting for the 2x coarsening, separably and with reuse:
// a thread owns coarse column (cx, cy) and marches PZC coarse layers up z.
// rc(cz) = P(2cz-1)/2 + P(2cz) + P(2cz+1)/2 with the fine-plane sums
// P(fz) = sum_dy w_dy (r(2cx-1)/2 + r(2cx) + r(2cx+1)/2) at row 2cy+dy; P(2cz+1)
// is kept for the next layer, and r(2cx-1) of a lane is r(2cx+1) of the lane
// below (a warp shuffle), so each fine value is loaded about 1.5 times.
constexpr int PZR = 4;
// UPD (mixed-precision CG): the residual update r -= alpha Ap of the finest
// level fused in.  rf is the old residual and Ap the product; each thread
// writes the updated values of the fine nodes its coarse cell owns (fine x, y,
// z in {2c, 2c + 1}) to rOut (a different vector: neighbouring cells read
// the old values of their halos) and sums their squares for r.r; halo values
// (row 2cy-1, the block's first plane, the left x neighbour of lane 0) are
// recomputed from rf and Ap.  checkDone = 2: run only in an iteration that
// replaced the residual by the true one (restricting the replacement).
template <typename T, bool UPD>
__global__ void __launch_bounds__(256) kRestrict2(Grid gf, Grid gc, const T* __restrict__ rf, const T* __restrict__ Ap,
                                                  T* __restrict__ rOut, T* __restrict__ rc, Scalars* S, RedBuf rb,
                                                  int checkDone) {
    if (checkDone && S->done) return;
    if (checkDone == 2 && S->replStamp != S->matvecs) return;
    const int lane = threadIdx.x;
    const int cx = blockIdx.x * 32 + lane, cy = blockIdx.y * 8 + threadIdx.y;
    const bool valid = cx < gc.nx && cy < gc.ny;
    const T half = T(0.5);
    const T av = UPD ? (T)S->alpha : T(0);
    const int fx0 = 2 * cx;
    DotAcc<T> acc;
    // Weighted plane sum at fine layer fz: the three rows 2cy-1 .. 2cy+1, each
    // r(2cx-1)/2 + r(2cx) + r(2cx+1)/2.  All loads of the plane are issued first,
    // then the shuffles; all lanes take part, out-of-grid fine nodes count 0.
    auto planeSum = [&](int fz, bool ownPlane, T (&P)[3]) {
        T c0[3][3], c1[3][3], cl[3][3];
        int64_t bases[3];
        bool ok0s[3], ok1s[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            const int fy = 2 * cy - 1 + r;
            const bool rowOk = fy >= 0 && fy < gf.ny && fz >= 0 && fz < gf.nz;
            const int64_t base = rowOk ? gf.store(0, fy, fz) : 0;
            const bool ok0 = rowOk && fx0 < gf.nx, ok1 = rowOk && fx0 + 1 < gf.nx;
            const bool okl = lane == 0 && rowOk && fx0 - 1 >= 0 && fx0 - 1 < gf.nx;
            bases[r] = base;
            ok0s[r] = ok0;
            ok1s[r] = ok1;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                c0[r][c] = ok0 ? rf[3 * (base + fx0) + c] : T(0);
                c1[r][c] = ok1 ? rf[3 * (base + fx0 + 1) + c] : T(0);
                cl[r][c] = okl ? rf[3 * (base + fx0 - 1) + c] : T(0);
                if (UPD) {
                    const T a0 = ok0 ? Ap[3 * (base + fx0) + c] : T(0);
                    const T a1 = ok1 ? Ap[3 * (base + fx0 + 1) + c] : T(0);
                    const T al = okl ? Ap[3 * (base + fx0 - 1) + c] : T(0);
                    c0[r][c] = fma(-av, a0, c0[r][c]);
                    c1[r][c] = fma(-av, a1, c1[r][c]);
                    cl[r][c] = fma(-av, al, cl[r][c]);
                }
            }
        }
        if (UPD && ownPlane && valid) {
#pragma unroll
            for (int r = 1; r < 3; ++r)
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    if (ok0s[r]) {
                        rOut[3 * (bases[r] + fx0) + c] = c0[r][c];
                        acc.add(c0[r][c] * c0[r][c]);
                    }
                    if (ok1s[r]) {
                        rOut[3 * (bases[r] + fx0 + 1) + c] = c1[r][c];
                        acc.add(c1[r][c] * c1[r][c]);
                    }
                }
        }
        T row[3][3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                T cm = __shfl_up_sync(0xffffffffu, c1[r][c], 1);
                if (lane == 0) cm = cl[r][c];
                row[r][c] = c0[r][c] + half * (cm + c1[r][c]);
            }
#pragma unroll
        for (int c = 0; c < 3; ++c) P[c] = row[1][c] + half * (row[0][c] + row[2][c]);
    };
    const int cz0 = blockIdx.z * PZR, cz1 = min(gc.nz, cz0 + PZR);
    T Pm[3];
    planeSum(2 * cz0 - 1, false, Pm);
    for (int cz = cz0; cz < cz1; ++cz) {
        T P0[3], Pp[3];
        planeSum(2 * cz, true, P0);
        planeSum(2 * cz + 1, true, Pp);
        if (valid) {
            T* q = rc + 3 * gc.store(cx, cy, cz);
#pragma unroll
            for (int c = 0; c < 3; ++c) q[c] = P0[c] + half * (Pm[c] + Pp[c]);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) Pm[c] = Pp[c];
    }
    if (UPD) {
        double v[1] = {acc.get()}, t[1];
        if (gridReduce<256, 1>(v, rb, t)) applyEpi(EPI_CONV, S, t[0], 0.0);
    }
}

template <typename T, int DIV>
__device__ __forceinline__ void prolongAt(const Grid& gf, const Grid& gc, const T* zc, int fx, int fy, int fz,
                                          T (&acc)[3]) {
    const int px = fx / DIV, py = fy / DIV, pz = fz / DIV;
    const int rx = fx - px * DIV, ry = fy - py * DIV, rz = fz - pz * DIV;
    const T inv = T(1) / T(DIV);
    acc[0] = acc[1] = acc[2] = T(0);
#pragma unroll
    for (int iz = 0; iz < 2; ++iz) {
        if (iz && rz == 0) continue;
        const T wz = iz ? T(rz) * inv : T(DIV - rz) * inv;
#pragma unroll
        for (int iy = 0; iy < 2; ++iy) {
            if (iy && ry == 0) continue;
            const T wy = iy ? T(ry) * inv : T(DIV - ry) * inv;
#pragma unroll
            for (int ix = 0; ix < 2; ++ix) {
                if (ix && rx == 0) continue;
                const T wx = ix ? T(rx) * inv : T(DIV - rx) * inv;
                const T w = wz * wy * wx;
                const T* p = zc + 3 * gc.store(px + ix, py + iy, pz + iz);
                acc[0] = fma(w, p[0], acc[0]);
                acc[1] = fma(w, p[1], acc[1]);
                acc[2] = fma(w, p[2], acc[2]);
            }
        }
    }
}

// Reference-mode up-leg of the V-cycle: zf = P zc + coef * dinv o rf on used
// nodes (coef = 2: the down-leg and up-leg Jacobi steps of the reference, which
// never update r), 0 elsewhere; fixed nodes zeroed on the finest level.
template <typename T, int DIV>
__global__ void __launch_bounds__(256)
    kProlongSmooth(Grid gf, Grid gc, const T* __restrict__ zc, const T* __restrict__ rf, const T* __restrict__ dinv,
                   const uint8_t* __restrict__ flags, T* __restrict__ zf, double coef, int maskFixed,
                   const T* __restrict__ aux, int epi, Scalars* S, RedBuf rb, int checkDone) {
    if (checkDone && S->done) return;
    const int fx = blockIdx.x * 32 + threadIdx.x, fy = blockIdx.y * 8 + threadIdx.y;
    const bool valid = fx < gf.nx && fy < gf.ny;
    DotAcc<T> d0, d1;
    if (valid) {
        for (int fz = blockIdx.z * PZ; fz < min(gf.nz, (int)(blockIdx.z + 1) * PZ); ++fz) {
            const int64_t s = gf.store(fx, fy, fz);
            const uint8_t fl = flags[s];
            T out[3] = {T(0), T(0), T(0)};
            T r[3] = {T(0), T(0), T(0)};
            if (fl & FLAG_USED) {
                T acc[3];
                prolongAt<T, DIV>(gf, gc, zc, fx, fy, fz, acc);
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    r[c] = rf[3 * s + c];
                    out[c] = acc[c] + (T)coef * dinv[3 * s + c] * r[c];
                }
                if (maskFixed && (fl & FLAG_FIXED)) out[0] = out[1] = out[2] = T(0);
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) zf[3 * s + c] = out[c];
            if (epi != EPI_NONE) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    d0.add(r[c] * out[c]);
                    if (aux) d1.add(out[c] * aux[3 * s + c]);
                }
            }
        }
    }
    if (epi != EPI_NONE) {
        double v[2] = {d0.get(), d1.get()}, t[2];
        if (gridReduce<256, 2>(v, rb, t)) applyEpi(epi, S, t[0], t[1]);
    }
}

// The same up-leg for the 2x coarsening, one thread per coarse cell column: a
// thread marches PZC coarse layers up z and writes the up-to-8 fine nodes
// (2cx+{0,1}, 2cy+{0,1}, 2cz+{0,1}) of each cell.  The coarse corners are read
// once per layer (the top corners become the next layer's bottom ones) and the
// trilinear weights are applied separably (z, then y, then x), so the kernel
// issues ~1.5 coarse loads per fine node instead of ~10.
constexpr int PZC = 4;
template <typename T>
__global__ void __launch_bounds__(256)
    kProlongSmooth2(Grid gf, Grid gc, const T* __restrict__ zc, const T* __restrict__ rf, const T* __restrict__ dinv,
                    const uint8_t* __restrict__ flags, T* __restrict__ zf, double coef, int maskFixed,
                    const T* __restrict__ aux, int epi, Scalars* S, RedBuf rb, int checkDone) {
    if (checkDone && S->done) return;
    const int cx = blockIdx.x * 32 + threadIdx.x, cy = blockIdx.y * 8 + threadIdx.y;
    // even fine x / y of the cell exist (the last coarse column has no fine node
    // when the fine element count is odd), and the odd ones
    const bool valid = cx < gc.nx && cy < gc.ny && 2 * cx < gf.nx && 2 * cy < gf.ny;
    const bool hx = valid && cx + 1 < gc.nx && 2 * cx + 1 < gf.nx;
    const bool hy = valid && cy + 1 < gc.ny && 2 * cy + 1 < gf.ny;
    const T half = T(0.5), cf = (T)coef;
    DotAcc<T> d0, d1;
    // Corner values of a coarse layer: [iy][ix][c], 0 where the corner does not exist.
    auto loadLayer = [&](int cz, T (&v)[2][2][3]) {
#pragma unroll
        for (int iy = 0; iy < 2; ++iy)
#pragma unroll
            for (int ix = 0; ix < 2; ++ix) {
                const bool ok = valid && cz < gc.nz && (ix == 0 || hx) && (iy == 0 || hy);
                v[iy][ix][0] = v[iy][ix][1] = v[iy][ix][2] = T(0);
                if (ok) {
                    const T* p = zc + 3 * gc.store(cx + ix, cy + iy, cz);
#pragma unroll
                    for (int c = 0; c < 3; ++c) v[iy][ix][c] = p[c];
                }
            }
    };
    // Fine layer fz from the plane values P at the cell's coarse corners.
    // All loads of a fine layer are issued before any is used (the flag does not
    // guard them: vectors hold 0 at unused nodes), so they overlap in flight.
    auto emit = [&](int fz, const T (&P)[2][2][3]) {
        T rr[2][2][3], dd[2][2][3];
        uint8_t ff[2][2];
#pragma unroll
        for (int jy = 0; jy < 2; ++jy)
#pragma unroll
            for (int jx = 0; jx < 2; ++jx) {
                const bool ex = (jx == 0 || hx) && (jy == 0 || hy);
                const int64_t s = ex ? gf.store(2 * cx + jx, 2 * cy + jy, fz) : 0;
                ff[jy][jx] = ex ? flags[s] : (uint8_t)0;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    rr[jy][jx][c] = ex ? rf[3 * s + c] : T(0);
                    dd[jy][jx][c] = ex ? dinv[3 * s + c] : T(0);
                }
            }
#pragma unroll
        for (int jy = 0; jy < 2; ++jy) {
            if (jy && !hy) continue;
#pragma unroll
            for (int jx = 0; jx < 2; ++jx) {
                if (jx && !hx) continue;
                const int64_t s = gf.store(2 * cx + jx, 2 * cy + jy, fz);
                const uint8_t fl = ff[jy][jx];
                const bool used = (fl & FLAG_USED) != 0;
                const bool zero = !used || (maskFixed && (fl & FLAG_FIXED));
                T out[3], r[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const T a0 = jx ? half * (P[0][0][c] + P[0][1][c]) : P[0][0][c];
                    const T a1 = jx ? half * (P[1][0][c] + P[1][1][c]) : P[1][0][c];
                    const T pv = jy ? half * (a0 + a1) : a0;
                    r[c] = used ? rr[jy][jx][c] : T(0);
                    out[c] = zero ? T(0) : pv + cf * dd[jy][jx][c] * r[c];
                    zf[3 * s + c] = out[c];
                }
                if (epi != EPI_NONE) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        d0.add(r[c] * out[c]);
                        if (aux) d1.add(out[c] * aux[3 * s + c]);
                    }
                }
            }
        }
    };
    if (valid) {
        const int cz0 = blockIdx.z * PZC, cz1 = min(gc.nz, cz0 + PZC);
        T B[2][2][3], Tp[2][2][3], M[2][2][3];
        loadLayer(cz0, B);
        for (int cz = cz0; cz < cz1; ++cz) {
            if (2 * cz >= gf.nz) break;
            const bool hz = cz + 1 < gc.nz && 2 * cz + 1 < gf.nz;
            emit(2 * cz, B);
            if (hz) {
                loadLayer(cz + 1, Tp);
#pragma unroll
                for (int iy = 0; iy < 2; ++iy)
#pragma unroll
                    for (int ix = 0; ix < 2; ++ix)
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            M[iy][ix][c] = half * (B[iy][ix][c] + Tp[iy][ix][c]);
                            B[iy][ix][c] = Tp[iy][ix][c];
                        }
                emit(2 * cz + 1, M);
            }
        }
    }
    if (epi != EPI_NONE) {
        double v[2] = {d0.get(), d1.get()}, t[2];
        if (gridReduce<256, 2>(v, rb, t)) applyEpi(epi, S, t[0], t[1]);
    }
}

template <typename T>
__global__ void __launch_bounds__(256) kJacobiZero(int64_t nnode, const T* __restrict__ r, const T* __restrict__ dinv,
                                                   const uint8_t* __restrict__ flags, T* __restrict__ z, double omega,
                                                   const Scalars* S, int checkDone) {
    if (checkDone && S->done) return;
    for (int64_t s = blockIdx.x * (int64_t)NT + threadIdx.x; s < nnode; s += (int64_t)gridDim.x * NT) {
        const uint8_t fl = flags[s];
        const bool act = (fl & FLAG_USED) && !(fl & FLAG_FIXED);
#pragma unroll
        for (int c = 0; c < 3; ++c) z[3 * s + c] = act ? (T)omega * dinv[3 * s + c] * r[3 * s + c] : T(0);
    }
}

template <typename T, int DIV>
__global__ void __launch_bounds__(256) kProlongAdd(Grid gf, Grid gc, const T* __restrict__ zc,
                                                   const uint8_t* __restrict__ flags, T* __restrict__ zf,
                                                   const Scalars* S, int checkDone) {
    if (checkDone && S->done) return;
    const int fx = blockIdx.x * 32 + threadIdx.x, fy = blockIdx.y * 8 + threadIdx.y;
    if (fx >= gf.nx || fy >= gf.ny) return;
    for (int fz = blockIdx.z * PZ; fz < min(gf.nz, (int)(blockIdx.z + 1) * PZ); ++fz) {
        const int64_t s = gf.store(fx, fy, fz);
        const uint8_t fl = flags[s];
        if (!(fl & FLAG_USED) || (fl & FLAG_FIXED)) continue;
        T acc[3];
        prolongAt<T, DIV>(gf, gc, zc, fx, fy, fz, acc);
#pragma unroll
        for (int c = 0; c < 3; ++c) zf[3 * s + c] += acc[c];
    }
}

template <typename T>
__global__ void kCoarseGather(int64_t n, const int32_t* __restrict__ freeDof, const T* __restrict__ rc,
                              T* __restrict__ b, const Scalars* S, int checkDone) {
    if (checkDone && S->done) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = rc[freeDof[i]];
}

// 4-wide vector loads/stores of the flat vector kernels (float4; two double2).
template <typename T>
struct V4;
template <>
struct V4<float> {
    static __device__ __forceinline__ void ld(const float* p, float (&v)[4]) {
        const float4 t = *reinterpret_cast<const float4*>(p);
        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    }
    static __device__ __forceinline__ void st(float* p, const float (&v)[4]) {
        *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
    }
};
template <>
struct V4<double> {
    static __device__ __forceinline__ void ld(const double* p, double (&v)[4]) {
        const double2 a = reinterpret_cast<const double2*>(p)[0], b = reinterpret_cast<const double2*>(p)[1];
        v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
    }
    static __device__ __forceinline__ void st(double* p, const double (&v)[4]) {
        reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
        reinterpret_cast<double2*>(p)[1] = make_double2(v[2], v[3]);
    }
};

// The 2x up-leg in flat form (same values as kProlongSmooth2): a block owns
// the fine rows [fy0, fy0 + PR) of fine layer fz, which are one contiguous
// range of every fine vector, and a thread takes 4 consecutive nodes at a time
// (12 values: three 16-byte loads of r and of dinv, three 16-byte stores of z,
// one 4-byte load of the flags).  The coarse rows the block interpolates from
// (PR/2 + 1 of them, averaged over the two coarse layers when fz is odd) are
// copied to shared memory with asynchronous copies while the first chunk
// loads, so a fine node costs 3-12 shared loads.  Only the first and last
// chunk of a block, which the neighbouring blocks share, take the scalar path
// (and every chunk when a vector is not 16-byte aligned).  Measured on GB300:
// 16 rows per block beat 32 (a partial last wave of blocks) and a persistent
// grid taking units from a counter (its per-unit barriers and counter round
// trips cost more than the wave tail).
constexpr int PR = 16;
constexpr int kProlongCoarseRows = PR / 2 + 1;
constexpr size_t kProlongFlatMaxSmem = 200 * 1024;
__host__ __device__ inline int prolongFlatRowGroups(const Grid& gf) { return (gf.ny + PR - 1) / PR; }

template <typename T>
__device__ __forceinline__ void cpAsync(T* dst, const T* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(d), "l"(src), "n"(sizeof(T)) : "memory");
}

// Inverse-diagonal values of a chunk: T, or FP16 (scaled; 8-byte loads).
__device__ __forceinline__ float diagVal(__half h) { return __half2float(h); }
__device__ __forceinline__ float diagVal(float v) { return v; }
__device__ __forceinline__ double diagVal(double v) { return v; }
template <typename T>
__device__ __forceinline__ void ldDiag12(const T* p, T (&v)[12]) {
#pragma unroll
    for (int q = 0; q < 3; ++q) V4<T>::ld(p + 4 * q, *reinterpret_cast<T(*)[4]>(v + 4 * q));
}
__device__ __forceinline__ void ldDiag12(const __half* p, float (&v)[12]) {
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const uint2 raw = reinterpret_cast<const uint2*>(p)[q];
        const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&raw.x));
        const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&raw.y));
        v[4 * q] = a.x;
        v[4 * q + 1] = a.y;
        v[4 * q + 2] = b.x;
        v[4 * q + 3] = b.y;
    }
}

// DT: the type the inverse diagonal is stored in (T, or FP16 scaled so that
// coef already carries the scale).
template <typename T, typename DT>
__global__ void __launch_bounds__(256)
    kProlongFlat(Grid gf, Grid gc, const T* __restrict__ zc, const T* __restrict__ rf, const DT* __restrict__ dinv,
                 const uint8_t* __restrict__ flags, T* __restrict__ zf, double coef, int maskFixed,
                 const T* __restrict__ aux, int epi, int vec, float invNx, Scalars* S, RedBuf rb, int checkDone) {
    if (checkDone && S->done) return;
    extern __shared__ __align__(16) unsigned char prolongSmem[];
    T* C = reinterpret_cast<T*>(prolongSmem);  // [kProlongCoarseRows][3 * gc.nx], then the layer above
    const int groups = prolongFlatRowGroups(gf);
    const int fz = blockIdx.x / groups;
    const int fy0 = (blockIdx.x - fz * groups) * PR, fy1 = min(gf.ny, fy0 + PR);
    const int cw = 3 * gc.nx, cy0 = fy0 >> 1, cz = fz >> 1;
    const int nstage = min(kProlongCoarseRows, gc.ny - cy0) * cw;
    const bool zodd = fz & 1;
    const T half = T(0.5), cf = (T)coef;
    {
        // the block's coarse rows are contiguous in each coarse layer
        const T* src = zc + 3 * gc.store(0, cy0, cz);
        const int64_t up = 3 * ((int64_t)gc.nx * gc.ny);
        for (int j = threadIdx.x; j < nstage; j += blockDim.x) {
            cpAsync(C + j, src + j);
            if (zodd) cpAsync(C + nstage + j, src + up + j);
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    }
    const int64_t nBeg = gf.store(0, fy0, fz);  // first node of the block
    const int nb = (fy1 - fy0) * gf.nx;
    const int64_t j1 = (nBeg + nb + 3) >> 2;
    DotAcc<T> d0, d1;
    // One chunk of 4 nodes; FULL: all 4 in the block's range and vectors aligned.
    auto chunk = [&](auto fullTag, int64_t n0, int ln0, const T (&rv)[12], const T (&dv)[12], uint32_t fl4) {
        constexpr bool FULL = decltype(fullTag)::value;
        // (ly, fx) of the chunk's first node; fx < 0 for nodes before the range
        const int lnc = max(ln0, 0);
        int ly = __float2int_rz(((float)lnc + 0.5f) * invNx);
        int fx = lnc - ly * gf.nx;
        if (fx < 0) { --ly; fx += gf.nx; }
        if (fx >= gf.nx) { ++ly; fx -= gf.nx; }
        fx -= lnc - ln0;
        T ov[12];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int ln = ln0 + t;
            const bool in = FULL || (ln >= 0 && ln < nb);
            if (in) {
                const uint32_t fl = (fl4 >> (8 * t)) & 0xffu;
                const bool used = (fl & FLAG_USED) != 0;
                const bool zero = !used || (maskFixed && (fl & FLAG_FIXED));
                const T* b = C + (ly >> 1) * cw + 3 * (fx >> 1);
                T pv[3];
                if (fx & 1) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) pv[c] = half * (b[c] + b[c + 3]);
                } else {
#pragma unroll
                    for (int c = 0; c < 3; ++c) pv[c] = b[c];
                }
                if (ly & 1) {
                    const T* b1 = b + cw;
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
                    const T r = used ? rv[3 * t + c] : T(0);
                    const T out = zero ? T(0) : pv[c] + cf * dv[3 * t + c] * r;
                    if (epi != EPI_NONE) {
                        d0.add(r * out);
                        if (aux) d1.add(out * aux[3 * (n0 + t) + c]);
                    }
                    if (FULL) ov[3 * t + c] = out;
                    else zf[3 * (n0 + t) + c] = out;
                }
            }
            if (++fx == gf.nx) {
                fx = 0;
                ++ly;
            }
        }
        if (FULL) {
#pragma unroll
            for (int v = 0; v < 3; ++v) V4<T>::st(zf + 3 * n0 + 4 * v, *reinterpret_cast<T(*)[4]>(ov + 4 * v));
        }
    };
    bool staged = false;
    for (int64_t j = (nBeg >> 2) + threadIdx.x;; j += blockDim.x) {
        const bool have = j < j1;
        const int64_t n0 = 4 * j;
        const int ln0 = (int)(n0 - nBeg);  // -3 .. nb - 1
        const bool full = vec && ln0 >= 0 && ln0 + 4 <= nb;
        T rv[12], dv[12];
        uint32_t fl4 = 0;
        if (have) {
            if (full) {
#pragma unroll
                for (int v = 0; v < 3; ++v) {
                    V4<T>::ld(rf + 3 * n0 + 4 * v, *reinterpret_cast<T(*)[4]>(rv + 4 * v));
                }
                ldDiag12(dinv + 3 * n0, dv);
                fl4 = *reinterpret_cast<const uint32_t*>(flags + n0);
            } else {
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const bool in = ln0 + t >= 0 && ln0 + t < nb;
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        rv[3 * t + c] = in ? rf[3 * (n0 + t) + c] : T(0);
                        dv[3 * t + c] = in ? (T)diagVal(dinv[3 * (n0 + t) + c]) : T(0);
                    }
                    if (in) fl4 |= (uint32_t)flags[n0 + t] << (8 * t);
                }
            }
        }
        if (!staged) {
            // every thread passes here once, after issuing its first chunk's loads
            asm volatile("cp.async.wait_all;\n" ::: "memory");
            __syncthreads();
            if (zodd) {
                for (int q = threadIdx.x; q < nstage; q += blockDim.x) C[q] = half * (C[q] + C[nstage + q]);
                __syncthreads();
            }
            staged = true;
        }
        if (!have) break;
        if (full) chunk(std::true_type{}, n0, ln0, rv, dv, fl4);
        else chunk(std::false_type{}, n0, ln0, rv, dv, fl4);
    }
    if (epi != EPI_NONE) {
        double v[2] = {d0.get(), d1.get()}, t[2];
        if (gridReduce<256, 2>(v, rb, t)) applyEpi(epi, S, t[0], t[1]);
    }
}

// y = Kinv b with the full inverse, one warp per row (FP64: the packed form below
// needs two FMAs per stored value plus FP64 shuffle reductions, which GB300's
// narrow FP64 pipe turns into 1.7x the time of this one-FMA-per-value form).
__global__ void __launch_bounds__(256) kGemv64(const double* __restrict__ K, int64_t n, const double* __restrict__ b,
                                               const int32_t* __restrict__ freeDof, double* __restrict__ zc,
                                               const Scalars* S, int checkDone) {
    if (checkDone && S->done) return;
    const int lane = threadIdx.x & 31;
    const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (row >= n) return;
    const double* k = K + row * n;
    double acc = 0.0;
    for (int64_t j = lane; j < n; j += 32) acc = fma(k[j], b[j], acc);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) zc[freeDof[row]] = acc;
}

// ---- coarsest solve of the mixed-precision cycle: y = Kinv b with the
// symmetric inverse stored once, in FP16.  Kinv is kept as the lower block
// triangle of 64 x 64 tiles (tile (I, J <= I) at index I (I + 1) / 2 + J,
// row-major inside, zero-padded past n), a quarter of the bytes of the full
// FP32 matrix.  The stored values are Kinv / scale with scale a power of two
// that maps the largest diagonal entry to 2^14 (|Kinv_ij| <= max diag for an
// SPD inverse), so every entry above 2^-10 of that maximum keeps FP16's 11-bit
// significand; the products accumulate in FP32.  The rounding is symmetric, so
// the coarse operator stays symmetric.  kSymRuns streams runs of consecutive
// tiles of one row block: it reads each tile once, accumulates K_IJ b_J for
// y_I over the run and writes K_IJ^T b_I (for y_J, off-diagonal tiles) per
// tile; kSymRunsReduce sums the partials per row block in a fixed order
// (deterministic, no atomics) and applies the scale.
__host__ __device__ inline int64_t symTileCount(int64_t nb) { return nb * (nb + 1) / 2; }
// Tile index -> (I, J): FP32 square root, corrected exactly in integers (an FP64
// square root per thread would run on GB300's narrow FP64 pipe).
__device__ inline void symTileDecode(int64_t t, int64_t& I, int64_t& J) {
    int64_t i = (int64_t)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
    while (i > 0 && i * (i + 1) / 2 > t) --i;
    while ((i + 1) * (i + 2) / 2 <= t) ++i;
    I = i;
    J = t - i * (i + 1) / 2;
}

__global__ void kPackSymHalf(const float* __restrict__ K, int64_t n, int64_t nb, float invScale,
                             __half* __restrict__ tiles) {
    const int64_t total = symTileCount(nb) * CT * CT;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t I, J;
        symTileDecode(i / (CT * CT), I, J);
        const int e = (int)(i % (CT * CT));
        const int64_t row = I * CT + e / CT, col = J * CT + e % CT;
        tiles[i] = __float2half_rn((row < n && col < n) ? K[row * n + col] * invScale : 0.0f);
    }
}

// *out = max |x_i| as FP32 bits (non-negative floats order like their bits); *out zeroed by the caller.
__global__ void __launch_bounds__(256) kMaxAbs(const float* __restrict__ x, int64_t n, unsigned* __restrict__ out) {
    float m = 0.0f;
    for (int64_t i = blockIdx.x * (int64_t)NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT) m = fmaxf(m, fabsf(x[i]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

__global__ void __launch_bounds__(256) kToHalf(const float* __restrict__ x, int64_t n, float invScale,
                                               __half* __restrict__ y) {
    for (int64_t i = blockIdx.x * (int64_t)NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT)
        y[i] = __float2half_rn(x[i] * invScale);
}

// Largest diagonal entry of a row-major n x n matrix (one block).
__global__ void __launch_bounds__(1024) kMaxDiag(const float* __restrict__ K, int64_t n, float* __restrict__ out) {
    __shared__ float red[32];
    float m = 0.0f;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) m = fmaxf(m, K[i * n + i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0) *out = m;
    }
}

// Runs of tiles: row block I's tiles are contiguous in memory; a run is up to
// SYM_RUN consecutive tiles (I, J0 .. J0 + SYM_RUN - 1) of one row, and one
// block streams a run.  Runs of row I: ceil((I + 1) / SYM_RUN), numbered in row
// order from symRunStart(I).
constexpr int SYM_RUN = 16;
__host__ __device__ inline int64_t symRunStart(int64_t I) {
    const int64_t a = I / SYM_RUN, b = I % SYM_RUN;
    return SYM_RUN * a * (a + 1) / 2 + b * (a + 1);
}

// One run per block, 16 x 16 threads each holding a 4 x 4 sub-block of every
// tile (four 8-byte row loads).  The row sums K_IJ b_J accumulate in registers across the
// run and reduce once (partial of the run at part[run][0..63]); the column sums
// K_IJ^T b_I of each off-diagonal tile reduce over the row groups through a
// double-buffered shared array (one barrier per tile) into part[tile][64..127].
// The next tile's values are loaded while the current one is used.
__global__ void __launch_bounds__(256) kSymRuns(const __half* __restrict__ tiles, const float* __restrict__ b,
                                                float* __restrict__ part, int64_t nb, const Scalars* S,
                                                int checkDone) {
    if (checkDone && S->done) return;
    __shared__ float colp[2][8][CT];
    const int64_t run = blockIdx.x;
    int64_t lo = 0, hi = nb - 1;  // largest I with symRunStart(I) <= run
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) / 2;
        if (symRunStart(mid) <= run) lo = mid;
        else hi = mid - 1;
    }
    const int64_t I = lo;
    const int64_t J0 = (run - symRunStart(I)) * SYM_RUN, J1 = min(J0 + SYM_RUN, I + 1);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tc = lane & 15, tr = warp * 2 + (lane >> 4);
    const int64_t rowTile = I * (I + 1) / 2;
    float bI[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) bI[j] = b[I * CT + 4 * tr + j];
    float rs[4] = {0.f, 0.f, 0.f, 0.f};
    uint2 nxt[4];
    auto loadTile = [&](int64_t J, uint2 (&raw)[4]) {
        const __half* K = tiles + (rowTile + J) * (CT * CT);
#pragma unroll
        for (int i = 0; i < 4; ++i) raw[i] = *reinterpret_cast<const uint2*>(K + (4 * tr + i) * CT + 4 * tc);
    };
    loadTile(J0, nxt);
    int buf = 0;
    for (int64_t J = J0; J < J1; ++J) {
        uint2 cur[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) cur[i] = nxt[i];
        if (J + 1 < J1) loadTile(J + 1, nxt);
        const float2 bJ01 = make_float2(b[J * CT + 4 * tc], b[J * CT + 4 * tc + 1]);
        const float2 bJ23 = make_float2(b[J * CT + 4 * tc + 2], b[J * CT + 4 * tc + 3]);
        float2 cs01 = make_float2(0.f, 0.f), cs23 = make_float2(0.f, 0.f);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float2 k01 = __half22float2(*reinterpret_cast<const __half2*>(&cur[i].x));
            const float2 k23 = __half22float2(*reinterpret_cast<const __half2*>(&cur[i].y));
            const float2 r2 = __ffma2_rn(k23, bJ23, __fmul2_rn(k01, bJ01));
            rs[i] += r2.x + r2.y;
            const float2 bi = make_float2(bI[i], bI[i]);
            cs01 = __ffma2_rn(k01, bi, cs01);
            cs23 = __ffma2_rn(k23, bi, cs23);
        }
        if (J != I) {  // the same for the whole block
            float cs[4] = {cs01.x, cs01.y, cs23.x, cs23.y};
#pragma unroll
            for (int j = 0; j < 4; ++j) cs[j] += __shfl_xor_sync(0xffffffffu, cs[j], 16);
            if (lane < 16) {
#pragma unroll
                for (int j = 0; j < 4; ++j) colp[buf][warp][4 * tc + j] = cs[j];
            }
            __syncthreads();
            if (threadIdx.x < CT) {
                float sum = 0.f;
#pragma unroll
                for (int w = 0; w < 8; ++w) sum += colp[buf][w][threadIdx.x];
                part[(rowTile + J) * (2 * CT) + CT + threadIdx.x] = sum;
            }
            buf ^= 1;
        }
    }
#pragma unroll
    for (int o = 1; o < 16; o <<= 1)
#pragma unroll
        for (int i = 0; i < 4; ++i) rs[i] += __shfl_xor_sync(0xffffffffu, rs[i], o);
    if (tc == 0) {
#pragma unroll
        for (int i = 0; i < 4; ++i) part[run * (2 * CT) + 4 * tr + i] = rs[i];
    }
}

// y_I = scale (sum over the runs of row I of their row partials + sum_{I' > I}
// (K_I'I^T b_I')), in a fixed order.
__global__ void __launch_bounds__(1024) kSymRunsReduce(const float* __restrict__ part, int64_t nb, int64_t n,
                                                       const int32_t* __restrict__ freeDof, float scale,
                                                       float* __restrict__ zc, const Scalars* S, int checkDone) {
    if (checkDone && S->done) return;
    __shared__ float red[16][CT];
    const int64_t I = blockIdx.x;
    const int r = threadIdx.x & (CT - 1), grp = threadIdx.x >> 6;
    float s = 0.f;
    for (int64_t q = symRunStart(I) + grp; q < symRunStart(I + 1); q += 16) s += part[q * (2 * CT) + r];
    for (int64_t Ip = I + 1 + grp; Ip < nb; Ip += 16) s += part[(Ip * (Ip + 1) / 2 + I) * (2 * CT) + CT + r];
    red[grp][r] = s;
    __syncthreads();
    if (grp == 0) {
        float y = 0.f;
#pragma unroll
        for (int q = 0; q < 16; ++q) y += red[q][r];
        const int64_t i = I * CT + r;
        if (i < n) zc[freeDof[i]] = y * scale;
    }
}

// x += alpha p; r -= alpha Ap; r.r.  TX = double is the FP64 solution; TX = float
// is the mixed-precision correction accumulated since the last flush.
template <typename TX, typename TV>
__global__ void __launch_bounds__(256) kUpdateXR(int64_t n, TX* __restrict__ x, TV* __restrict__ r,
                                                 const TV* __restrict__ p, const TV* __restrict__ Ap, Scalars* S,
                                                 RedBuf rb) {
    if (S->done) return;
    const TX ax = (TX)S->alpha;
    const TV av = (TV)S->alpha;
    DotAcc<TV> acc;
    const int64_t tid = blockIdx.x * (int64_t)NT + threadIdx.x, stride = (int64_t)gridDim.x * NT;
    const int64_t n4 = n / 4;
    for (int64_t q = tid; q < n4; q += stride) {
        TX xv[4];
        TV rv[4], pv[4], av4[4];
        V4<TX>::ld(x + 4 * q, xv);
        V4<TV>::ld(r + 4 * q, rv);
        V4<TV>::ld(p + 4 * q, pv);
        V4<TV>::ld(Ap + 4 * q, av4);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            xv[k] = fma(ax, (TX)pv[k], xv[k]);
            rv[k] = fma(-av, av4[k], rv[k]);
            acc.add(rv[k] * rv[k]);
        }
        V4<TX>::st(x + 4 * q, xv);
        V4<TV>::st(r + 4 * q, rv);
    }
    for (int64_t i = 4 * n4 + tid; i < n; i += stride) {
        x[i] = fma(ax, (TX)p[i], x[i]);
        const TV ri = fma(-av, Ap[i], r[i]);
        r[i] = ri;
        acc.add(ri * ri);
    }
    double v[1] = {acc.get()}, t[1];
    if (gridReduce<NT, 1>(v, rb, t)) applyEpi(EPI_CONV, S, t[0], 0.0);
}

// Mixed precision: r -= alpha Ap; r.r.  The solution update x += alpha p of
// the same iteration is deferred to kUpdatePX (or kFlushX), which read p anyway.
__global__ void __launch_bounds__(256) kUpdateR(int64_t n, float* __restrict__ r, const float* __restrict__ Ap,
                                                Scalars* S, RedBuf rb) {
    if (S->done) return;
    const float av = (float)S->alpha;
    DotAcc<float> acc;
    const int64_t tid = blockIdx.x * (int64_t)NT + threadIdx.x, stride = (int64_t)gridDim.x * NT;
    const int64_t n4 = n / 4;
    for (int64_t q = tid; q < n4; q += stride) {
        float rv[4], av4[4];
        V4<float>::ld(r + 4 * q, rv);
        V4<float>::ld(Ap + 4 * q, av4);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            rv[k] = fma(-av, av4[k], rv[k]);
            acc.add(rv[k] * rv[k]);
        }
        V4<float>::st(r + 4 * q, rv);
    }
    for (int64_t i = 4 * n4 + tid; i < n; i += stride) {
        const float ri = fma(-av, Ap[i], r[i]);
        r[i] = ri;
        acc.add(ri * ri);
    }
    double v[1] = {acc.get()}, t[1];
    if (gridReduce<NT, 1>(v, rb, t)) applyEpi(EPI_CONV, S, t[0], 0.0);
}

// Mixed precision: fold the FP32 solution correction, and this iteration's
// deferred alpha p, into the FP64 solution.  conditional = 1: only when an FP64
// true-residual pass follows in this iteration (kUpdateR has run, so alpha p is
// pending; the stamp tells kUpdatePX it is folded).  conditional = 0 (after the
// last iteration): alpha p only if kUpdateR ran in the last iteration and
// neither a flush nor kUpdatePX has folded it.
__global__ void __launch_bounds__(256) kFlushX(int64_t n, double* __restrict__ x64, float* __restrict__ x32,
                                               const float* __restrict__ pFirst, const float* __restrict__ pSecond,
                                               Scalars* S, int conditional) {
    if (conditional && (S->done || !trueResidualDue(S))) return;
    const float* __restrict__ p = S->pSel ? pSecond : pFirst;
    const bool pending =
        conditional || (S->rStamp == S->matvecs && S->foldStamp != S->matvecs && S->pxStamp != S->matvecs);
    const double a = pending ? S->alpha : 0.0;
    for (int64_t i = blockIdx.x * (int64_t)NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT) {
        x64[i] += (double)x32[i] + a * (double)p[i];
        x32[i] = 0.f;
    }
    if (conditional && blockIdx.x == 0 && threadIdx.x == 0) S->foldStamp = S->matvecs;
}

// Mixed precision: p = z + beta p, and the deferred x += alpha p (old p) of
// this iteration unless a flush has folded it.
__global__ void __launch_bounds__(256) kUpdatePX(int64_t n, float* __restrict__ p, const float* __restrict__ z,
                                                 float* __restrict__ x, Scalars* S) {
    if (S->done) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) S->pxStamp = S->matvecs;  // read only by kFlushX
    const float beta = (float)S->beta;
    const float ax = S->foldStamp == S->matvecs ? 0.f : (float)S->alpha;
    const int64_t tid = blockIdx.x * (int64_t)NT + threadIdx.x, stride = (int64_t)gridDim.x * NT;
    const int64_t n4 = n / 4;
    for (int64_t q = tid; q < n4; q += stride) {
        float pv[4], zv[4], xv[4];
        V4<float>::ld(p + 4 * q, pv);
        V4<float>::ld(z + 4 * q, zv);
        V4<float>::ld(x + 4 * q, xv);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            xv[k] = fma(ax, pv[k], xv[k]);
            pv[k] = fma(beta, pv[k], zv[k]);
        }
        V4<float>::st(p + 4 * q, pv);
        V4<float>::st(x + 4 * q, xv);
    }
    for (int64_t i = 4 * n4 + tid; i < n; i += stride) {
        x[i] = fma(ax, p[i], x[i]);
        p[i] = fma(beta, p[i], z[i]);
    }
}

template <typename T>
__global__ void __launch_bounds__(256) kUpdateP(int64_t n, T* __restrict__ p, const T* __restrict__ z,
                                                const Scalars* S, int first) {
    if (S->done) return;
    const T beta = first ? T(0) : (T)S->beta;
    const int64_t tid = blockIdx.x * (int64_t)NT + threadIdx.x, stride = (int64_t)gridDim.x * NT;
    const int64_t n4 = n / 4;
    for (int64_t q = tid; q < n4; q += stride) {
        T pv[4], zv[4];
        V4<T>::ld(p + 4 * q, pv);
        V4<T>::ld(z + 4 * q, zv);
#pragma unroll
        for (int k = 0; k < 4; ++k) pv[k] = fma(beta, pv[k], zv[k]);
        V4<T>::st(p + 4 * q, pv);
    }
    for (int64_t i = 4 * n4 + tid; i < n; i += stride) p[i] = fma(beta, p[i], z[i]);
}

template <typename T>
__global__ void __launch_bounds__(256) kDots(int64_t n, const T* __restrict__ a, const T* __restrict__ b,
                                             const T* __restrict__ c, const T* __restrict__ d, int epi, Scalars* S,
                                             RedBuf rb, int checkDone) {
    if (checkDone && S->done) return;
    DotAcc<T> s0, s1;
    for (int64_t i = blockIdx.x * (int64_t)NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT) {
        if (a) s0.add(a[i] * b[i]);
        if (c) s1.add(c[i] * d[i]);
    }
    double v[2] = {s0.get(), s1.get()}, t[2];
    if (gridReduce<NT, 2>(v, rb, t)) applyEpi(epi, S, t[0], t[1]);
}

// Deflation coarse space, part 1: t_j = v_j . r - (K v_j) . z (j < k; z may be
// null), reduced over the grid; the last block stores G^-1 t in the solver scalars.
template <typename T>
__global__ void __launch_bounds__(256) kCoarseDots(int64_t n, int k, const T* __restrict__ V,
                                                   const T* __restrict__ KV, const T* __restrict__ r,
                                                   const T* __restrict__ z, CoarseSpace G, Scalars* S, RedBuf rb,
                                                   int checkDone) {
    if (checkDone && S->done) return;
    DotAcc<T> acc[4];
    for (int64_t i = blockIdx.x * (int64_t)NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT) {
        const T ri = r[i];
        const T zi = z ? z[i] : T(0);
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (j < k) {
                acc[j].add(V[(int64_t)j * n + i] * ri);
                if (z) acc[j].add(-KV[(int64_t)j * n + i] * zi);
            }
    }
    double v[4] = {acc[0].get(), acc[1].get(), acc[2].get(), acc[3].get()}, t[4];
    if (gridReduce<NT, 4>(v, rb, t)) {
        for (int a = 0; a < 4; ++a) {
            double sum = 0.0;
            for (int b = 0; b < k; ++b) sum += G.Ginv[4 * a + b] * t[b];
            S->coarseCoef[a] = a < k ? sum : 0.0;
        }
    }
}

// Part 2: z += sum_j coef_j v_j.
template <typename T>
__global__ void __launch_bounds__(256) kCoarseAxpy(int64_t n, int k, const T* __restrict__ V, T* __restrict__ z,
                                                   const Scalars* S, int checkDone) {
    if (checkDone && S->done) return;
    T cf[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) cf[j] = (T)S->coarseCoef[j];
    for (int64_t i = blockIdx.x * (int64_t)NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT) {
        T zi = z[i];
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (j < k) zi = fma(cf[j], V[(int64_t)j * n + i], zi);
        z[i] = zi;
    }
}

// Start projection: x += sum_j mu_j v_j, r -= sum_j mu_j (K v_j).
__global__ void __launch_bounds__(256) kCoarseStart(int64_t n, int k, const double* __restrict__ V,
                                                    const double* __restrict__ KV, const Scalars* S,
                                                    double* __restrict__ x, double* __restrict__ r) {
    double mu[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) mu[j] = S->coarseCoef[j];
    for (int64_t i = blockIdx.x * (int64_t)NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT) {
        double xi = x[i], ri = r[i];
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (j < k) {
                xi = fma(mu[j], V[(int64_t)j * n + i], xi);
                ri = fma(-mu[j], KV[(int64_t)j * n + i], ri);
            }
        x[i] = xi;
        r[i] = ri;
    }
}

template <typename TI, typename TO>
__global__ void kConvert(int64_t n, const TI* __restrict__ x, TO* __restrict__ y) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = (TO)x[i];
}

template <typename T>
__global__ void kFill(int64_t n, T* __restrict__ y, T v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = v;
}

template <typename T>
__global__ void kScatterCompressed(int64_t nn, const int32_t* __restrict__ store, const double* __restrict__ comp,
                                   T* __restrict__ dense, unsigned* bad) {
    bool ok = true;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < 3 * nn; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = comp[i];
        ok = ok && isfinite(v);
        dense[3 * (int64_t)store[i / 3] + i % 3] = (T)v;
    }
    if (bad && !ok) atomicOr(bad, 1u);
}

template <typename T>
__global__ void kGatherCompressed(int64_t nn, const int32_t* __restrict__ store, const T* __restrict__ dense,
                                  double* __restrict__ comp) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < 3 * nn; i += (int64_t)gridDim.x * blockDim.x)
        comp[i] = (double)dense[3 * (int64_t)store[i / 3] + i % 3];
}

// One parity colour of the coarsest-matrix assembly: same-colour elements share
// no node, so plain += is race-free and the summation order is fixed.
template <typename T>
__global__ void kAssembleCoarse(Grid g, const float* __restrict__ E, const int32_t* __restrict__ freeNode,
                                const Kd<double> ke, double scale, T* __restrict__ K, int64_t n, int color) {
    const int hx = (g.ex + 1 - (color & 1)) / 2, hy = (g.ey + 1 - ((color >> 1) & 1)) / 2;
    const int64_t e = blockIdx.x;
    const int ix = (int)(e % hx), iy = (int)((e / hx) % hy), iz = (int)(e / ((int64_t)hx * hy));
    const int x = 2 * ix + (color & 1), y = 2 * iy + ((color >> 1) & 1), z = 2 * iz + (color >> 2);
    if (x >= g.ex || y >= g.ey || z >= g.ez) return;
    const float Ee = E[g.store(x, y, z)];
    if (Ee == 0.f) return;
    for (int ent = threadIdx.x; ent < 576; ent += blockDim.x) {
        const int r = ent / 24, c = ent % 24;
        const int a = r / 3, ci = r % 3, b = c / 3, cj = c % 3;
        const int32_t na = freeNode[g.store(x + (a & 1), y + ((a >> 1) & 1), z + (a >> 2))];
        const int32_t nb = freeNode[g.store(x + (b & 1), y + ((b >> 1) & 1), z + (b >> 2))];
        if (na < 0 || nb < 0) continue;
        K[(3 * (int64_t)na + ci) * n + 3 * (int64_t)nb + cj] += (T)(scale * (double)Ee * ke.v[ent]);
    }
}

template <typename T>
__global__ void kSymmetrize(T* K, int64_t n) {
    // Column-major lower triangle (cuSOLVER) == row-major upper triangle: copy it down.
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n * n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / n, c = i % n;
        if (c < r) K[i] = K[c * n + r];
    }
}

__global__ void kInitScalars(Scalars* S, double tol, long long maxIter, int flexible, int mixed, int replaceEvery,
                             double delta, int breakAt) {
    Scalars s = {};
    s.breakAt = breakAt;
    s.tol2 = tol * tol;
    s.maxIter = maxIter;
    s.flexible = flexible;
    s.mixed = mixed;
    s.replaceEvery = replaceEvery;
    s.delta2 = mixed ? delta * delta : 0.0;
    s.rStamp = s.foldStamp = s.pxStamp = s.replStamp = -1;
    *S = s;
}

inline int flatBlocks(int64_t n) {
    int64_t b = (n + NT - 1) / NT;
    if (b > 152 * 8) b = 152 * 8;
    if (b < 1) b = 1;
    return (int)b;
}

inline dim3 nodeGrid(const Grid& g) {
    return dim3((g.nx + 31) / 32, (g.ny + 7) / 8, (g.nz + PZ - 1) / PZ);
}

}  // namespace

// ------------------------------------------------------------------ launchers

cudaError_t setKernelAttributes() {
    const int s64 = (kSuElems + kSyElems) * (int)sizeof(double), s32 = (kSuElems + kSyElems) * (int)sizeof(float);
    const int sdf = (kSuElems + kSyElems) * (int)sizeof(df);
    const cudaFuncAttribute A = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(kMatvecH<double, double>, A, s64))) return e;
    if ((e = cudaFuncSetAttribute(kMatvecH<float, float>, A, s32))) return e;
    if ((e = cudaFuncSetAttribute(kMatvecH<float, float, OUT_CG>, A, s32))) return e;
    if ((e = cudaFuncSetAttribute(kMatvecH<float, float, OUT_CG_PX>, A, s32))) return e;
    if ((e = cudaFuncSetAttribute(kMatvecH<double, double, OUT_CG>, A, s64))) return e;
    if ((e = cudaFuncSetAttribute(kMatvecH<double, df, OUT_TRUE>, A, sdf))) return e;
    if ((e = cudaFuncSetAttribute(kMatvecH<double, df>, A, sdf))) return e;
    if ((e = cudaFuncSetAttribute(kMatvec<double>, A, s64))) return e;
    if ((e = cudaFuncSetAttribute(kMatvec<float>, A, s32))) return e;
    return cudaFuncSetAttribute(kMatvec<double, df>, A, sdf);
}

template <typename T>
int launchMatvec(const LaunchCtx& c, const MatvecArgs<T>& a, bool structured, const void* opconst) {
    const Grid& g = a.g;
    dim3 grid((g.nx + MV_TX - 2) / (MV_TX - 1), (g.ny + MV_TY - 2) / (MV_TY - 1), (g.nz + MV_ZC - 1) / MV_ZC);
    dim3 block(MV_TX, MV_TY);
    size_t smem = (size_t)(kSuElems + kSyElems) * sizeof(T);
    if (structured) {
        Ks<T> k;
        const T* src = static_cast<const T*>(opconst);
        for (int i = 0; i < 45; ++i) k.v[i] = src[i];
        if (a.mode == MV_AX && a.dot0 == DOT_X_OUT && !a.dot1 && !a.y32)
            kMatvecH<T, T, OUT_CG><<<grid, block, smem, c.stream>>>(a, k, c.S, c.rb);
        else
            kMatvecH<T, T><<<grid, block, smem, c.stream>>>(a, k, c.S, c.rb);
    } else {
        Kd<T> k;
        const T* src = static_cast<const T*>(opconst) + 45;
        for (int i = 0; i < 576; ++i) k.v[i] = src[i];
        kMatvec<T><<<grid, block, smem, c.stream>>>(a, k, c.S, c.rb);
    }
    return 1;
}

int launchMatvecPX(const LaunchCtx& c, const MatvecArgs<float>& a, const float* opconst) {
    const Grid& g = a.g;
    dim3 grid((g.nx + MV_TX - 2) / (MV_TX - 1), (g.ny + MV_TY - 2) / (MV_TY - 1), (g.nz + MV_ZC - 1) / MV_ZC);
    dim3 block(MV_TX, MV_TY);
    size_t smem = (size_t)(kSuElems + kSyElems) * sizeof(float);
    Ks<float> k;
    for (int i = 0; i < 45; ++i) k.v[i] = opconst[i];
    kMatvecH<float, float, OUT_CG_PX><<<grid, block, smem, c.stream>>>(a, k, c.S, c.rb);
    return 1;
}

int launchMatvecDF(const LaunchCtx& c, const MatvecArgs<double>& a, bool structured, const double* opconst) {
    const Grid& g = a.g;
    dim3 grid((g.nx + MV_TX - 2) / (MV_TX - 1), (g.ny + MV_TY - 2) / (MV_TY - 1), (g.nz + MV_ZC - 1) / MV_ZC);
    dim3 block(MV_TX, MV_TY);
    size_t smem = (size_t)(kSuElems + kSyElems) * sizeof(df);
    if (structured) {
        Ks<df> k;
        for (int i = 0; i < 45; ++i) k.v[i] = df(opconst[i]);
        if (a.mode == MV_RESID && a.dot0 == DOT_OUT_OUT && !a.dot1 && a.y32)
            kMatvecH<double, df, OUT_TRUE><<<grid, block, smem, c.stream>>>(a, k, c.S, c.rb);
        else
            kMatvecH<double, df><<<grid, block, smem, c.stream>>>(a, k, c.S, c.rb);
    } else {
        Kd<df> k;
        for (int i = 0; i < 576; ++i) k.v[i] = df(opconst[45 + i]);
        kMatvec<double, df><<<grid, block, smem, c.stream>>>(a, k, c.S, c.rb);
    }
    return 1;
}

template <typename T>
int launchRestrict(const LaunchCtx& c, const Grid& gf, const Grid& gc, int div, const T* rf, T* rc, int checkDone) {
    dim3 block(32, 8);
    if (div == 4) {
        kRestrict<T, 4><<<nodeGrid(gc), block, 0, c.stream>>>(gf, gc, rf, rc, c.S, checkDone);
    } else {
        if constexpr (std::is_same<T, float>::value) {
            if ((c.tma & 1) && launchRestrictTma(c, gf, gc, rf, nullptr, nullptr, rc, checkDone)) return 1;
        }
        dim3 grid((gc.nx + 31) / 32, (gc.ny + 7) / 8, (gc.nz + PZR - 1) / PZR);
        kRestrict2<T, false><<<grid, block, 0, c.stream>>>(gf, gc, rf, nullptr, nullptr, rc, c.S, c.rb, checkDone);
    }
    return 1;
}

int launchUpdateRestrict(const LaunchCtx& c, const Grid& gf, const Grid& gc, const float* rIn, const float* Ap,
                         float* rOut, float* rc) {
    if ((c.tma & 1) && launchRestrictTma(c, gf, gc, rIn, Ap, rOut, rc, 1)) return 1;
    dim3 block(32, 8), grid((gc.nx + 31) / 32, (gc.ny + 7) / 8, (gc.nz + PZR - 1) / PZR);
    kRestrict2<float, true><<<grid, block, 0, c.stream>>>(gf, gc, rIn, Ap, rOut, rc, c.S, c.rb, 1);
    return 1;
}

template <typename T>
int launchProlongSmooth(const LaunchCtx& c, const Grid& gf, const Grid& gc, int div, const T* zc, const T* rf,
                        const T* dinv, const uint8_t* flags, T* zf, double coef, int maskFixed, const T* aux, int epi,
                        int checkDone, HalfDiag hd) {
    dim3 grid = nodeGrid(gf), block(32, 8);
    const int64_t flatBlocksN = (int64_t)prolongFlatRowGroups(gf) * gf.nz;
    const size_t flatSmem = 2 * sizeof(T) * kProlongCoarseRows * 3 * (size_t)gc.nx;
    if (div == 2 && flatBlocksN <= kMaxRedBlocks && flatSmem <= kProlongFlatMaxSmem) {
        auto al = [](const void* q) { return ((uintptr_t)q & 15u) == 0; };
        const bool half = std::is_same<T, float>::value && hd.d != nullptr;
        const int vec = al(rf) && al(zf) && ((uintptr_t)flags & 3u) == 0 &&
                        (half ? ((uintptr_t)hd.d & 7u) == 0 : al(dinv));
        auto go = [&](auto kern, const auto* dptr, double cf) {
            if (flatSmem > 48 * 1024)
                cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kProlongFlatMaxSmem);
            kern<<<(unsigned)flatBlocksN, 256, flatSmem, c.stream>>>(gf, gc, zc, rf, dptr, flags, zf, cf, maskFixed, aux,
                                                                     epi, vec, 1.0f / gf.nx, c.S, c.rb, checkDone);
        };
        if constexpr (std::is_same<T, float>::value) {
            if (half) {
                if ((c.tma & 2) && launchProlongBulk(c, gf, gc, zc, rf, hd.d, flags, zf, coef * (double)hd.scale, maskFixed,
                                               aux, epi, checkDone))
                    return 1;
                go(kProlongFlat<float, __half>, hd.d, coef * (double)hd.scale);
                return 1;
            }
        }
        go(kProlongFlat<T, T>, dinv, coef);
    } else if (div == 2) {
        // grids beyond the flat kernel's block or shared-memory limits (over ~1000^3 nodes)
        dim3 cgrid((gc.nx + 31) / 32, (gc.ny + 7) / 8, (gc.nz + PZC - 1) / PZC);
        kProlongSmooth2<T><<<cgrid, block, 0, c.stream>>>(gf, gc, zc, rf, dinv, flags, zf, coef, maskFixed, aux, epi,
                                                          c.S, c.rb, checkDone);
    } else if (div == 4)
        kProlongSmooth<T, 4><<<grid, block, 0, c.stream>>>(gf, gc, zc, rf, dinv, flags, zf, coef, maskFixed, aux, epi,
                                                             c.S, c.rb, checkDone);
    else
        kProlongSmooth<T, 2><<<grid, block, 0, c.stream>>>(gf, gc, zc, rf, dinv, flags, zf, coef, maskFixed, aux, epi,
                                                             c.S, c.rb, checkDone);
    return 1;
}

template <typename T>
int launchJacobiZero(const LaunchCtx& c, const Grid& g, const T* r, const T* dinv, const uint8_t* flags, T* z,
                     double omega, int checkDone) {
    kJacobiZero<T><<<flatBlocks(g.nnode), NT, 0, c.stream>>>(g.nnode, r, dinv, flags, z, omega, c.S, checkDone);
    return 1;
}

template <typename T>
int launchProlongAdd(const LaunchCtx& c, const Grid& gf, const Grid& gc, int div, const T* zc, const uint8_t* flags,
                     T* zf, int checkDone) {
    dim3 grid = nodeGrid(gf), block(32, 8);
    if (div == 4) kProlongAdd<T, 4><<<grid, block, 0, c.stream>>>(gf, gc, zc, flags, zf, c.S, checkDone);
    else kProlongAdd<T, 2><<<grid, block, 0, c.stream>>>(gf, gc, zc, flags, zf, c.S, checkDone);
    return 1;
}

template <typename T>
int launchCoarseSolve(const LaunchCtx& c, CoarseInv<T> Kinv, int64_t n, const int32_t* freeDof, const T* rc, T* tmp,
                      T* part, T* zc, int checkDone) {
    if (n <= 0) return 0;
    kCoarseGather<T><<<(int)((n + 255) / 256), 256, 0, c.stream>>>(n, freeDof, rc, tmp, c.S, checkDone);
    if constexpr (std::is_same<T, double>::value) {
        kGemv64<<<(int)((n * 32 + 255) / 256), 256, 0, c.stream>>>(Kinv.K, n, tmp, freeDof, zc, c.S, checkDone);
        return 2;
    } else {
        const int64_t nb = coarseBlocks(n);
        kSymRuns<<<(unsigned)symRunStart(nb), 256, 0, c.stream>>>(Kinv.K, tmp, part, nb, c.S, checkDone);
        kSymRunsReduce<<<(unsigned)nb, 1024, 0, c.stream>>>(part, nb, n, freeDof, Kinv.scale, zc, c.S, checkDone);
        return 3;
    }
}

int launchMaxAbs(cudaStream_t s, const float* x, int64_t n, unsigned* outBits) {
    kMaxAbs<<<flatBlocks(n), NT, 0, s>>>(x, n, outBits);
    return 1;
}

int launchToHalf(cudaStream_t s, const float* x, int64_t n, float invScale, __half* y) {
    kToHalf<<<flatBlocks(n), NT, 0, s>>>(x, n, invScale, y);
    return 1;
}

int launchMaxDiag(cudaStream_t s, const float* K, int64_t n, float* out) {
    kMaxDiag<<<1, 1024, 0, s>>>(K, n, out);
    return 1;
}

int launchPackSymHalf(cudaStream_t s, const float* K, int64_t n, float invScale, __half* tiles) {
    const int64_t nb = coarseBlocks(n);
    kPackSymHalf<<<flatBlocks(symTileCount(nb) * CT * CT), NT, 0, s>>>(K, n, nb, invScale, tiles);
    return 1;
}

template <typename TX, typename TV>
int launchUpdateXR(const LaunchCtx& c, int64_t n, TX* x, TV* r, const TV* p, const TV* Ap) {
    kUpdateXR<TX, TV><<<flatBlocks(n), NT, 0, c.stream>>>(n, x, r, p, Ap, c.S, c.rb);
    return 1;
}

int launchFlushX(const LaunchCtx& c, int64_t n, double* x64, float* x32, const float* p, const float* pAlt,
                 int conditional) {
    kFlushX<<<flatBlocks(n), NT, 0, c.stream>>>(n, x64, x32, p, pAlt ? pAlt : p, c.S, conditional);
    return 1;
}

int launchUpdateR(const LaunchCtx& c, int64_t n, float* r, const float* Ap) {
    kUpdateR<<<flatBlocks(n), NT, 0, c.stream>>>(n, r, Ap, c.S, c.rb);
    return 1;
}

int launchUpdatePX(const LaunchCtx& c, int64_t n, float* p, const float* z, float* x) {
    kUpdatePX<<<flatBlocks(n), NT, 0, c.stream>>>(n, p, z, x, c.S);
    return 1;
}

template <typename T>
int launchUpdateP(const LaunchCtx& c, int64_t n, T* p, const T* z, int first) {
    kUpdateP<T><<<flatBlocks(n), NT, 0, c.stream>>>(n, p, z, c.S, first);
    return 1;
}

template <typename T>
int launchDots(const LaunchCtx& c, int64_t n, const T* a, const T* b, const T* cc, const T* d, int epi, int checkDone) {
    kDots<T><<<flatBlocks(n), NT, 0, c.stream>>>(n, a, b, cc, d, epi, c.S, c.rb, checkDone);
    return 1;
}

template <typename T>
int launchCoarseSpace(const LaunchCtx& c, int64_t n, int k, const T* V, const T* KV, const CoarseSpace& G,
                      const T* r, T* z, int checkDone) {
    kCoarseDots<T><<<flatBlocks(n), NT, 0, c.stream>>>(n, k, V, KV, r, z, G, c.S, c.rb, checkDone);
    kCoarseAxpy<T><<<flatBlocks(n), NT, 0, c.stream>>>(n, k, V, z, c.S, checkDone);
    return 2;
}

int launchCoarseStart(const LaunchCtx& c, int64_t n, int k, const double* V, const double* KV, const CoarseSpace& G,
                      double* x, double* r) {
    kCoarseDots<double><<<flatBlocks(n), NT, 0, c.stream>>>(n, k, V, KV, r, nullptr, G, c.S, c.rb, 0);
    kCoarseStart<<<flatBlocks(n), NT, 0, c.stream>>>(n, k, V, KV, c.S, x, r);
    return 2;
}

template <typename TI, typename TO>
int launchConvert(cudaStream_t s, int64_t n, const TI* x, TO* y) {
    kConvert<TI, TO><<<flatBlocks(n), NT, 0, s>>>(n, x, y);
    return 1;
}

template <typename T>
int launchFill(cudaStream_t s, int64_t n, T* y, T v) {
    kFill<T><<<flatBlocks(n), NT, 0, s>>>(n, y, v);
    return 1;
}

template <typename T>
int launchScatterCompressed(cudaStream_t s, int64_t nn, const int32_t* store, const double* comp, T* dense,
                            unsigned* bad) {
    kScatterCompressed<T><<<flatBlocks(3 * nn), NT, 0, s>>>(nn, store, comp, dense, bad);
    return 1;
}

template <typename T>
int launchGatherCompressed(cudaStream_t s, int64_t nn, const int32_t* store, const T* dense, double* comp) {
    kGatherCompressed<T><<<flatBlocks(3 * nn), NT, 0, s>>>(nn, store, dense, comp);
    return 1;
}

template <typename T>
int launchAssembleCoarse(cudaStream_t s, const Grid& g, const float* E, const int32_t* freeNode, const double* Ke,
                         double scale, T* K, int64_t n) {
    Kd<double> k;
    for (int i = 0; i < 576; ++i) k.v[i] = Ke[i];
    int launches = 0;
    for (int color = 0; color < 8; ++color) {
        const int hx = (g.ex + 1 - (color & 1)) / 2, hy = (g.ey + 1 - ((color >> 1) & 1)) / 2,
                  hz = (g.ez + 1 - (color >> 2)) / 2;
        const int64_t ne = (int64_t)hx * hy * hz;
        if (ne <= 0) continue;
        kAssembleCoarse<T><<<(unsigned)ne, 64, 0, s>>>(g, E, freeNode, k, scale, K, n, color);
        ++launches;
    }
    return launches;
}

template <typename T>
__global__ void kZeroStrictRowMajorLower(T* K, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n * n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / n, c = i - r * n;
        if (c < r) K[i] = T(0);
    }
}

template <typename T>
int launchZeroStrictRowMajorLower(cudaStream_t s, T* K, int64_t n) {
    kZeroStrictRowMajorLower<T><<<flatBlocks(n * n), NT, 0, s>>>(K, n);
    return 1;
}

template <typename T>
int launchSymmetrizeLowerToFull(cudaStream_t s, T* K, int64_t n) {
    kSymmetrize<T><<<flatBlocks(n * n), NT, 0, s>>>(K, n);
    return 1;
}

int launchInitScalars(cudaStream_t s, Scalars* S, double tol, long long maxIter, int flexible, int mixed,
                      int replaceEvery, double replaceDelta, int breakAt) {
    kInitScalars<<<1, 1, 0, s>>>(S, tol, maxIter, flexible, mixed, replaceEvery, replaceDelta, breakAt);
    return 1;
}

// ------------------------------------------------------------------ no-allocation product
//
// Scratch of vfem_apply_operator_device_noalloc: the reduction partials, the
// ticket and the scalar block of the fused x.(Kx) dot live in this file-scope
// device array instead of memory from cudaMalloc.  Fixed size: 2 x 65,536 block
// partials + 1 KiB (1,049,600 bytes); every GPU that loads the library holds it
// until the process exits.  All calls share it, so calls that overlap on the GPU
// race; each call clears the ticket and scalars before its kernel.
namespace {
// Partials of the product's grid reduction, which carries two sums per block
// (x.(Kx) and the unused second dot).
constexpr size_t kNoAllocPartialBytes = 2 * (size_t)kMaxRedBlocks * sizeof(double);
constexpr size_t kNoAllocBytes = kNoAllocPartialBytes + 1024;
static_assert(sizeof(Scalars) + 256 <= 1024, "scalar block does not fit the no-allocation scratch");
__device__ __align__(256) unsigned char g_noallocScratch[kNoAllocBytes];
std::mutex g_noallocMutex;
constexpr int kNoAllocMaxDevices = 64;
void* g_noallocAddr[kNoAllocMaxDevices] = {};
}  // namespace

cudaError_t noallocScratchSetup() {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_noallocMutex);
    if (g_noallocAddr[dev]) return cudaSuccess;
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noallocScratch);  // the host-side name is not a device address
    if (e != cudaSuccess) return e;
    g_noallocAddr[dev] = ptr;
    return cudaSuccess;
}

cudaError_t launchMatvecNoAlloc(cudaStream_t s, const MatvecArgs<double>& a, bool structured, const void* opconst,
                                double* xKx, bool* tooLarge) {
    const Grid& g = a.g;
    dim3 grid((g.nx + MV_TX - 2) / (MV_TX - 1), (g.ny + MV_TY - 2) / (MV_TY - 1), (g.nz + MV_ZC - 1) / MV_ZC);
    *tooLarge = (int64_t)grid.x * grid.y * grid.z > kMaxRedBlocks;
    if (*tooLarge) return cudaSuccess;
    cudaError_t e = noallocScratchSetup();
    if (e != cudaSuccess) return e;
    int dev = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    unsigned char* base = static_cast<unsigned char*>(g_noallocAddr[dev]);
    RedBuf rb{reinterpret_cast<double*>(base), reinterpret_cast<unsigned*>(base + kNoAllocPartialBytes)};
    Scalars* S = reinterpret_cast<Scalars*>(base + kNoAllocPartialBytes + 256);
    // The ticket and the scalars must start at zero; the partials are overwritten.
    if ((e = cudaMemsetAsync(base + kNoAllocPartialBytes, 0, 1024, s)) != cudaSuccess) return e;
    MatvecArgs<double> b = a;
    b.mode = MV_AX;
    b.dot0 = DOT_X_OUT;
    b.dot1 = 0;
    b.epi = EPI_STORE;
    b.checkDone = 0;
    b.condTrue = 0;
    size_t smem = (size_t)(kSuElems + kSyElems) * sizeof(double);
    dim3 block(MV_TX, MV_TY);
    if (structured) {
        Ks<double> k;
        for (int i = 0; i < 45; ++i) k.v[i] = static_cast<const double*>(opconst)[i];
        kMatvecH<double, double><<<grid, block, smem, s>>>(b, k, S, rb);
    } else {
        Kd<double> k;
        for (int i = 0; i < 576; ++i) k.v[i] = static_cast<const double*>(opconst)[45 + i];
        kMatvec<double><<<grid, block, smem, s>>>(b, k, S, rb);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    return cudaMemcpyAsync(xKx, &S->red0, sizeof(double), cudaMemcpyDeviceToDevice, s);
}

// ------------------------------------------------------------------ instantiations
#define INST_T(T)                                                                                                     \
    template int launchMatvec<T>(const LaunchCtx&, const MatvecArgs<T>&, bool, const void*);                         \
    template int launchRestrict<T>(const LaunchCtx&, const Grid&, const Grid&, int, const T*, T*, int);               \
    template int launchProlongSmooth<T>(const LaunchCtx&, const Grid&, const Grid&, int, const T*, const T*,          \
                                        const T*, const uint8_t*, T*, double, int, const T*, int, int, HalfDiag);    \
    template int launchJacobiZero<T>(const LaunchCtx&, const Grid&, const T*, const T*, const uint8_t*, T*, double,  \
                                     int);                                                                           \
    template int launchProlongAdd<T>(const LaunchCtx&, const Grid&, const Grid&, int, const T*, const uint8_t*, T*,  \
                                     int);                                                                           \
    template int launchCoarseSolve<T>(const LaunchCtx&, CoarseInv<T>, int64_t, const int32_t*, const T*, T*, T*,    \
                                      T*, int);                                                                      \
    template int launchUpdateP<T>(const LaunchCtx&, int64_t, T*, const T*, int);                                     \
    template int launchCoarseSpace<T>(const LaunchCtx&, int64_t, int, const T*, const T*, const CoarseSpace&, const T*, T*, int); \
    template int launchDots<T>(const LaunchCtx&, int64_t, const T*, const T*, const T*, const T*, int, int);         \
    template int launchFill<T>(cudaStream_t, int64_t, T*, T);                                                        \
    template int launchScatterCompressed<T>(cudaStream_t, int64_t, const int32_t*, const double*, T*, unsigned*);    \
    template int launchGatherCompressed<T>(cudaStream_t, int64_t, const int32_t*, const T*, double*);               \
    template int launchAssembleCoarse<T>(cudaStream_t, const Grid&, const float*, const int32_t*, const double*,     \
                                         double, T*, int64_t);                                                       \
    template int launchSymmetrizeLowerToFull<T>(cudaStream_t, T*, int64_t);                                          \
    template int launchZeroStrictRowMajorLower<T>(cudaStream_t, T*, int64_t);
INST_T(double)
INST_T(float)
template int launchUpdateXR<double, double>(const LaunchCtx&, int64_t, double*, double*, const double*, const double*);
template int launchConvert<double, float>(cudaStream_t, int64_t, const double*, float*);
template int launchConvert<float, double>(cudaStream_t, int64_t, const float*, double*);
template int launchConvert<double, double>(cudaStream_t, int64_t, const double*, double*);
template int launchConvert<float, float>(cudaStream_t, int64_t, const float*, float*);

}  // namespace vfem
