// Time per tcgen05.mma (kind::f16, BF16 operands from shared memory, FP32
// accumulator in tensor memory, M = 128, K = 16) for N = 32, 64, 128, 256,
// issued back to back by one thread; one CTA on one SM.  Prints, per N and
// batch size, the issue time and the time to completion (tcgen05.commit on an
// mbarrier, bounded wait) per MMA.  Exit status 1 if a batch did not complete.
// Used by tests/test_gpu_tensor_core.py.
#include <cstdint>
#include <cstdio>

__device__ __forceinline__ uint32_t smemU32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint64_t desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

template <int N>
__global__ void __launch_bounds__(128, 1) rate(int reps, long long* out) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int i = tid; i < 65536 / 4; i += 128) reinterpret_cast<uint32_t*>(sm)[i] = 0x3f803f80u;  // BF16 1.0
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smemU32(&mbar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smemU32(&tslot)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tb = tslot, smb = smemU32(sm);
    if (tid == 0) {
        const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((128u >> 4) << 24);
        // A: 16 row groups x 512 B + 512 B (< 9.1 KB from the start, at most 896 B
        // further on); B at 32 KB: N / 8 row groups x 256 B + 128 B; D at column 0 or 256.
        const uint64_t ad = desc(smb, 512, 512), bd = desc(smb + 32768, 128, 256);
        long long t0, t1, t2;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
        for (int r = 0; r < reps; ++r) {
            const uint32_t acc = r > 0;
            asm volatile(
                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tb + (uint32_t)((r & 1) * 256)),
                "l"(ad + (uint64_t)((r & 7) * 8)), "l"(bd), "r"(idesc), "r"(acc));
        }
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smemU32(&mbar)));
        uint32_t done = 0;
        for (long it = 0; it < 50000000 && !done; ++it)
            asm volatile(
                "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
                : "=r"(done)
                : "r"(smemU32(&mbar)));
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t2));
        out[0] = t1 - t0;
        out[1] = t2 - t0;
        out[2] = done;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tb));
}

template <int N>
bool run(long long* d) {
    cudaFuncSetAttribute(rate<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, 65536);
    bool ok = true;
    for (int reps : {24, 240, 2400}) {
        rate<N><<<1, 128, 65536>>>(reps, d);
        const cudaError_t e = cudaDeviceSynchronize();
        long long h[3] = {0, 0, 0};
        cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
        printf("N=%3d reps=%5d issue %9.1f ns (%6.1f ns/mma)  complete %9.1f ns (%6.1f ns/mma) done=%lld %s\n", N, reps,
               (double)h[0], (double)h[0] / reps, (double)h[1], (double)h[1] / reps, h[2], cudaGetErrorString(e));
        ok = ok && e == cudaSuccess && h[2] == 1;
    }
    return ok;
}

int main() {
    long long* d = nullptr;
    if (cudaMalloc(&d, 64) != cudaSuccess) return 1;
    const bool ok = run<32>(d) && run<64>(d) && run<128>(d) && run<256>(d);
    cudaFree(d);
    return ok ? 0 : 1;
}
