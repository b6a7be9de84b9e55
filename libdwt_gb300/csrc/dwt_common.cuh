// Shared device helpers of the GB300 lifting kernels: lifting parameters,
// symmetric-extension index mapping, exact (non-contracted) float arithmetic,
// and thin inline-PTX wrappers for mbarriers and the TMA bulk-copy engine.
#pragma once

#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

namespace dwt {

// Lifting parameters of one wavelet, in the order the steps are applied.
//
// Forward: steps c[0..n) alternate odd, even, odd, even samples; then even
// samples are multiplied by zeta_e and odd ones by zeta_o.
// Inverse: even samples are multiplied by zeta_o and odd ones by zeta_e; then
// steps c[0..n) alternate even, odd, even, odd samples.
// A signal of length 1 is only scaled: by n1 (n1_fwd / n1_inv).
//
// CDF 9/7 (src/libdwt.c:541-547, 5543, 5811):
//   forward (-p1, u1, -p2, u2), zeta_e = s1, zeta_o = 1/s1 rounded as a float
//   division; inverse (-u2, p2, -u1, p1); n1_inv = the constant s2.
// CDF 5/3 (src/libdwt.c:566-569, 5571-5592, 5838-5864):
//   forward (-p1, u1), zeta_e = s1, zeta_o = s2; inverse (-u1, p1).
struct Wavelet {
    float c[4];
    float zeta_e, zeta_o;
    float n1_fwd, n1_inv;
    int nsteps;
};

enum WaveletId { CDF97 = 0, CDF53 = 1 };

// The parameters of wavelet `id` (CDF97 / CDF53) for one direction.  Usable
// on the host and in device code; 1/zeta is a correctly rounded float
// division in both.
__host__ __device__ inline Wavelet make_wavelet_dev(int id, bool inverse)
{
    Wavelet w{};
    if (id == CDF97) {
        // src/libdwt.c:541-547
        const float p1 = 1.58613434342059f, u1 = -0.0529801185729f;
        const float p2 = -0.8829110755309f, u2 = 0.4435068520439f;
        const float s1 = 1.1496043988602f;
        const float s2 = (float)(1 / 1.1496043988602);
        w.nsteps = 4;
        w.zeta_e = s1;
        w.zeta_o = 1.0f / s1;
        w.n1_fwd = s1;
        w.n1_inv = s2;
        if (!inverse) {
            w.c[0] = -p1; w.c[1] = u1; w.c[2] = -p2; w.c[3] = u2;
        } else {
            w.c[0] = -u2; w.c[1] = p2; w.c[2] = -u1; w.c[3] = p1;
        }
    } else {
        // src/libdwt.c:566-569
        const float p1 = 0.5f, u1 = 0.25f;
        const float s1 = (float)1.41421356237309504880, s2 = (float)0.70710678118654752440;
        w.nsteps = 2;
        w.zeta_e = s1;
        w.zeta_o = s2;
        w.n1_fwd = s1;
        w.n1_inv = s2;
        if (!inverse) {
            w.c[0] = -p1; w.c[1] = u1;
        } else {
            w.c[0] = -u1; w.c[1] = p1;
        }
        w.c[2] = w.c[3] = 0.0f;
    }
    return w;
}

// Host-side construction for kernel launches.
Wavelet make_wavelet(int id, bool inverse);

// Exact IEEE single operations that the compiler may not fuse into an FMA.
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
// x + c*(l + r), three separately rounded operations.
__device__ __forceinline__ float lift(float x, float c, float l, float r)
{
    return fadd(x, fmul(c, fadd(l, r)));
}

// Two floats in one 64-bit register pair.  Additions use the packed FP32x2
// instruction of sm_100-class GPUs (add.rn.f32x2 rounds each half exactly as
// add.rn.f32 does); multiplications stay scalar mul.rn.f32.  A packed
// multiply that feeds a packed add is contracted into a fused multiply-add by
// the code generator even with explicit .rn rounding and --fmad=false (one
// rounding instead of two), which would break bit parity with the
// reference; scalar mul.rn.f32 is never contracted.
typedef unsigned long long f2;

__device__ __forceinline__ f2 pk(float lo, float hi)
{
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ float f2lo(f2 v)
{
    float a, b;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
    return a;
}
__device__ __forceinline__ float f2hi(f2 v)
{
    float a, b;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
    return b;
}
#ifndef DWT_SCALAR_PAIRS
__device__ __forceinline__ f2 add2(f2 a, f2 b)
{
    f2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
#else
__device__ __forceinline__ f2 add2(f2 a, f2 b)
{
    return pk(__fadd_rn(f2lo(a), f2lo(b)), __fadd_rn(f2hi(a), f2hi(b)));
}
#endif
__device__ __forceinline__ f2 mul2(f2 a, f2 b)
{
    return pk(__fmul_rn(f2lo(a), f2lo(b)), __fmul_rn(f2hi(a), f2hi(b)));
}
// x + c*(l + r) on both halves
__device__ __forceinline__ f2 lift2(f2 x, f2 c, f2 l, f2 r) { return add2(x, mul2(c, add2(l, r))); }

// Whole-sample symmetric extension of index r into [0, n), n >= 2: the
// periodic reflection with period 2(n-1).  Keeps the parity of r.
__host__ __device__ __forceinline__ int mirror(int r, int n)
{
    if (n <= 1) return 0;
    const int p = 2 * (n - 1);
    int m = r % p;
    if (m < 0) m += p;
    return (m >= n) ? p - m : m;
}

__host__ __device__ __forceinline__ int ceil_div(int a, int b) { return (a + b - 1) / b; }
__host__ __device__ __forceinline__ int ceil_div_pow2(int i, int j) { return (i + (1 << j) - 1) >> j; }

// ---------------------------------------------------------------- PTX wrappers

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}

// Plain arrival (count 1, release semantics), e.g. a consumer releasing a
// stage it has read.
__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait on an mbarrier phase.  try_wait itself suspends for a
// hardware-chosen interval, so the iteration cap is seconds of wall time.
constexpr uint32_t kWaitLimit = 1u << 24;

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint32_t limit = kWaitLimit)
{
    for (uint32_t i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// TMA tensor copy of one 2D box (the map's box shape) at element coordinates
// (x, y) to shared memory; completion signalled on `bar` as bytes.  `dst`
// must be 128-byte aligned and x * 4 bytes a multiple of 16.
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(smem_addr(dst)),
        "l"(map), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

// TMA bulk copy global -> shared, completion signalled on `bar` as bytes.
// dst and src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// Acquire load of a counter another warp releases (atomicAdd after a
// __threadfence), and the fence that orders the generic-proxy accesses seen
// so far before this thread's later TMA (async-proxy) accesses.
__device__ __forceinline__ int ld_acquire(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Release increment of a counter another warp acquires: the writes this
// thread has made (and those of the warp ordered before it by a warp
// barrier) are visible to an acquirer that sees the increment.
__device__ __forceinline__ void red_release_add(int *p, int v)
{
    asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ void fence_proxy_async_global()
{
    asm volatile("fence.proxy.async.global;" ::: "memory");
}

// TMA bulk copy shared -> global in the thread's bulk async-group; commit
// closes the group; wait_read<N> waits until at most N groups still read
// shared memory; wait_all until every group has completed its writes.
// Addresses 16-byte aligned, sizes multiples of 16 bytes.
__device__ __forceinline__ void bulk_s2g(void *dst, const void *src, uint32_t bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_addr(src)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void bulk_wait_read()
{
    asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Error codes raised by device code into the error word.
enum DeviceError : int {
    kErrNone = 0,
    kErrWaitTimeout = 1,   // an mbarrier wait gave up
    kErrQueueTimeout = 2,  // a work-queue dependency wait gave up (batch phases, ordered in-place units)
};

// Programmatic dependent launch.  A kernel launched by launch_pdl may be
// scheduled while its predecessor in the stream is still draining; it calls
// pdl_wait() before touching global memory (the wait returns once the
// predecessor has completed and its writes are visible) and pdl_release()
// to let its own successor start launching.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Whether level kernels are chained with programmatic dependent launch
// (default on; DWT_GPU_PDL=0 turns it off).
bool pdl_enabled();

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args... args)
{
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = pdl_enabled() ? 1 : 0;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

}  // namespace dwt
