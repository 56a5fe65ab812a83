// Device helpers shared by the tiled step kernels: packed FP32x2 arithmetic, mbarrier and
// bulk-copy PTX wrappers with bounded waits, storage-format loads, and the BFL wall rows.
#pragma once

#include <cstdint>

#include "step_common.cuh"

namespace islbm {
namespace {

// packed FP32 pair arithmetic (fma.rn.f32x2)
struct P2 { unsigned long long v; };
__device__ __forceinline__ P2 p2(float lo, float hi) {
    P2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ P2 p2(float2 a) { return p2(a.x, a.y); }
__device__ __forceinline__ void fma2(P2 &acc, P2 a, P2 b) {
    asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(acc.v) : "l"(a.v), "l"(b.v));
}
__device__ __forceinline__ float2 unp(P2 a) {
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(a.v));
    return r;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: gives up after about a second, records the fault and lets the kernel run
// to its end (no thread can be left behind at a barrier). Returns whether the phase completed.
// After one timeout the thread stops waiting altogether (`faulted`), so a broken pipeline
// costs one bounded wait, not one per plane; the CTA then starts no further copies and, at the
// end of the kernel, thread 0 waits (bounded again) for the copy phases still pending.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity, Ctrl *ctrl, bool &faulted) {
    if (faulted) return false;
    for (int it = 0; it < (1 << 22); ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if (it > 32) __nanosleep(256);
    }
    faulted = true;
    atomicOr(&ctrl->fault, 1u);
    return false;
}

// Pipeline word kept by every thread: bit s = parity of the next completion of stage s;
// bit PEND + s = (thread 0) a copy phase was posted on stage s and not yet seen complete;
// bit PPAR + s = the completion parity of that copy.
constexpr int PEND = 8, PPAR = 16;
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// Tensor memory (TMEM) used as per-thread storage: thread t of warp w owns lane 32*(w % 4) + t
// of the CTA's allocation; the warp-collective loads and stores below address the warp's lane
// quarter (`ta` = allocation base + (32*(w % 4) << 16) + column). Loads complete asynchronously:
// tmem_wait_ld ties the loaded registers, so no use of them is scheduled before the wait.
__device__ __forceinline__ void tmem_alloc(uint32_t *dst_smem, unsigned ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, unsigned ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmem_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void tmem_st8(uint32_t ta, float a0, float a1, float a2, float a3, float a4, float a5,
                                         float a6, float a7) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(ta),
                 "r"(__float_as_uint(a0)), "r"(__float_as_uint(a1)), "r"(__float_as_uint(a2)), "r"(__float_as_uint(a3)),
                 "r"(__float_as_uint(a4)), "r"(__float_as_uint(a5)), "r"(__float_as_uint(a6)), "r"(__float_as_uint(a7))
                 : "memory");
}
__device__ __forceinline__ void tmem_st2(uint32_t ta, float a0, float a1) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x2.b32 [%0], {%1, %2};" ::"r"(ta), "r"(__float_as_uint(a0)),
                 "r"(__float_as_uint(a1))
                 : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t ta, uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(ta)
        : "memory");
}
__device__ __forceinline__ void tmem_ld2(uint32_t ta, uint32_t (&v)[2]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0, %1}, [%2];" : "=r"(v[0]), "=r"(v[1]) : "r"(ta) : "memory");
}
// wait for this thread's TMEM loads; the registers of `a` and `b` are tied to the wait
__device__ __forceinline__ void tmem_wait_ld(uint32_t (&a)[16], uint32_t (&b)[16]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(a[0]), "+r"(a[1]), "+r"(a[2]), "+r"(a[3]), "+r"(a[4]), "+r"(a[5]), "+r"(a[6]), "+r"(a[7]),
                   "+r"(a[8]), "+r"(a[9]), "+r"(a[10]), "+r"(a[11]), "+r"(a[12]), "+r"(a[13]), "+r"(a[14]), "+r"(a[15]),
                   "+r"(b[0]), "+r"(b[1]), "+r"(b[2]), "+r"(b[3]), "+r"(b[4]), "+r"(b[5]), "+r"(b[6]), "+r"(b[7]),
                   "+r"(b[8]), "+r"(b[9]), "+r"(b[10]), "+r"(b[11]), "+r"(b[12]), "+r"(b[13]), "+r"(b[14]), "+r"(b[15])
                 :
                 : "memory");
}
__device__ __forceinline__ void tmem_wait_ld(uint32_t (&a)[16]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(a[0]), "+r"(a[1]), "+r"(a[2]), "+r"(a[3]), "+r"(a[4]), "+r"(a[5]), "+r"(a[6]), "+r"(a[7]),
                   "+r"(a[8]), "+r"(a[9]), "+r"(a[10]), "+r"(a[11]), "+r"(a[12]), "+r"(a[13]), "+r"(a[14]), "+r"(a[15])
                 :
                 : "memory");
}
// ties registers loaded before a tied wait: each empty volatile statement stays after that wait
// and redefines its register, so no use of it is scheduled earlier
template <int N> __device__ __forceinline__ void tmem_tie(uint32_t (&v)[N]) {
#pragma unroll
    for (int i = 0; i < N; i++) asm volatile("" : "+r"(v[i]));
}
__device__ __forceinline__ void tmem_wait_ld(uint32_t (&a)[2]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;" : "+r"(a[0]), "+r"(a[1]) : : "memory");
}

// four consecutive stored values -> float (deviation formats add the reference state `w`)
template <class S> __device__ __forceinline__ float4 ld4(const S *p, float w);
template <> __device__ __forceinline__ float4 ld4<float>(const float *p, float) { return *(const float4 *)p; }
template <> __device__ __forceinline__ float4 ld4<__half>(const __half *p, float w) {
    const uint2 r = *(const uint2 *)p;
    const float2 a = __half22float2(*(const __half2 *)&r.x), b = __half22float2(*(const __half2 *)&r.y);
    return make_float4(a.x + w, a.y + w, b.x + w, b.y + w);
}
template <> __device__ __forceinline__ float4 ld4<__nv_bfloat16>(const __nv_bfloat16 *p, float w) {
    const uint2 r = *(const uint2 *)p;
    const float2 a = __bfloat1622float2(*(const __nv_bfloat162 *)&r.x), b = __bfloat1622float2(*(const __nv_bfloat162 *)&r.y);
    return make_float4(a.x + w, a.y + w, b.x + w, b.y + w);
}
template <class S> __device__ __forceinline__ float ld1(const S *p, float w) {
    if constexpr (Storage<S>::dev) return to_c(*p) + w; else return (float)*p;
}
// stored value as it is (the deviation f - ref for the deviation formats): the interpolation
// weights of every filter sum to one, so filtering deviations and adding w once at the target
// equals filtering full values up to rounding
template <class S> __device__ __forceinline__ float ldv(const S *p) { return (float)to_c(*p); }
template <class S> __device__ __forceinline__ float2 ldv2(const S *p);
template <> __device__ __forceinline__ float2 ldv2<float>(const float *p) { return *(const float2 *)p; }
template <> __device__ __forceinline__ float2 ldv2<__half>(const __half *p) { return __half22float2(*(const __half2 *)p); }
template <> __device__ __forceinline__ float2 ldv2<__nv_bfloat16>(const __nv_bfloat16 *p) {
    return __bfloat1622float2(*(const __nv_bfloat162 *)p);
}
__device__ __forceinline__ float4 ld4(const float *p) { return *(const float4 *)p; }

__device__ __forceinline__ int wrapi(int v, int n) {
    v %= n;
    return v < 0 ? v + n : v;
}

// BFL rows (C/evolution.h:505-572) for one node, reading the old populations from global
// memory; rare (flagged wall rows only), kept out of line.
template <class S>
__device__ __forceinline__ void bfl_node_body(const S *__restrict__ fo, const Tables<float> &T, const StepConst &k, int x,
                                              int y, int z, float *F) {
    const int NX = k.NX, NY = k.NY;
    const size_t N = (size_t)NX*NY*k.NZ;
    const int nb = 2*k.NYD6;
    const int r = z*k.NYD6 + (y + 3);
    const int ix = k.bfl_mode ? r : x + 3;
    const int iy = k.bfl_mode ? r : y + 3;
    auto f = [&](int q, int xx, int yy, int zz) -> float {
        return load_f<S>(fo + (size_t)q*N, ((size_t)zz*NY + wrapi(yy, NY))*NX + wrapi(xx, NX), q);
    };
    auto bw = [&](int s, int a, int idx) -> float { return idx < nb ? T.bfl_w[((size_t)s*7 + a)*nb + idx] : 0.f; };
    auto y_xi = [&](int q, int sy, int sz) -> float {
        float outer = 0.f;
        for (int c = 0; c < 7; c++) {
            float in = f(q, x, y - 3, c)*bw(sy, 0, iy);
            for (int b = 1; b < 7; b++) in = in + f(q, x, y - 3 + b, c)*bw(sy, b, iy);
            outer = c == 0 ? in*bw(sz, 0, r) : outer + in*bw(sz, c, r);
        }
        return outer;
    };
    auto xy_xi = [&](int q, int sx, int sy, int sz) -> float {
        float outer = 0.f;
        for (int c = 0; c < 7; c++) {
            float mid = 0.f;
            for (int b = 0; b < 7; b++) {
                float in = f(q, x - 3, y - 3 + b, c)*bw(sx, 0, ix);
                for (int a = 1; a < 7; a++) in = in + f(q, x - 3 + a, y - 3 + b, c)*bw(sx, a, ix);
                mid = b == 0 ? in*bw(sy, 0, iy) : mid + in*bw(sy, b, iy);
            }
            outer = c == 0 ? mid*bw(sz, 0, r) : outer + mid*bw(sz, c, r);
        }
        return outer;
    };
    auto lin = [&](float q, int a, int b) -> float {
        return (1.f/(2.f*q))*f(a, x, y, z) + ((2.f*q - 1.f)/(2.f*q))*f(b, x, y, z);
    };
    if (T.bfl_flag[0*nb + r] == 1) {
        const float q = T.bfl_q[0*nb + r];
        if (q > 0.5f) { F[3] = lin(q, 4, 3); F[7] = lin(q, 10, 7); F[8] = lin(q, 9, 8); }
        if (q < 0.5f) { F[3] = y_xi(4, B_YB378, B_XIB378); F[7] = xy_xi(10, B_XB37, B_YB378, B_XIB378); F[8] = xy_xi(9, B_XB38, B_YB378, B_XIB378); }
    }
    if (T.bfl_flag[1*nb + r] == 1) {
        const float q = T.bfl_q[1*nb + r];
        if (q > 0.5f) { F[4] = lin(q, 3, 4); F[9] = lin(q, 8, 9); F[10] = lin(q, 7, 10); }
        if (q < 0.5f) { F[4] = y_xi(3, B_YB4910, B_XIB4910); F[9] = xy_xi(8, B_XB49, B_YB4910, B_XIB4910); F[10] = xy_xi(7, B_XB410, B_YB4910, B_XIB4910); }
    }
    if (T.bfl_flag[2*nb + r] == 1) {
        const float q = T.bfl_q[2*nb + r];
        if (q > 0.5f) F[15] = lin(q, 18, 15);
        if (q < 0.5f) F[15] = y_xi(18, B_YB15, B_XIB15);
    }
    if (T.bfl_flag[3*nb + r] == 1) {
        const float q = T.bfl_q[3*nb + r];
        if (q > 0.5f) F[16] = lin(q, 17, 16);
        if (q < 0.5f) F[16] = y_xi(17, B_YB16, B_XIB16);
    }
}

// out of line for callers that keep it off their hot path
template <class S>
__device__ __noinline__ void bfl_node(const S *__restrict__ fo, const Tables<float> &T, const StepConst &k, int x, int y, int z,
                                      float *F) {
    bfl_node_body<S>(fo, T, k, x, y, z, F);
}

}  // namespace
}  // namespace islbm
