// Tiled step kernel: z-marching x-y tiles staged in shared memory by bulk async copies.
//
// Same step as stream_collide (C/evolution.h:358-684) for FP32 arithmetic with FP32, FP16 or
// BF16 population storage, organised for HBM:
//   * a CTA owns a tile of TY full-width rows (all NX spanwise nodes, TY streamwise rows) and
//     marches upward through the wall-normal planes; every plane of the 18 moving
//     populations is copied global -> shared with cp.async.bulk (one copy per population and
//     plane, 3-row streamwise halo for the ten populations with e_y != 0, periodic wrap by
//     splitting the copy), tracked by an mbarrier, 3 stages deep;
//   * the interpolation is applied as separable filters, exact in real arithmetic because the
//     x and y weights are the same for every node (uniform spacing, C/initialization.h:51-108)
//     and the xi weights depend only on the target (y, z): a streamwise filter over the halo
//     rows, then a spanwise filter (4 nodes per task) through shared memory, then the xi
//     combination over a 7-plane ring of filtered values kept in registers, so each loaded
//     value feeds 7 target planes without being re-read;
//   * the collision tail, wall bounce-back, BFL rows and controller partial sums are fused;
//   * CTAs are persistent (one per SM) and split the flattened (tile, z) work evenly; a
//     segment that starts inside a column first re-reads the 6 planes below it.
// Every value of the old populations is read from HBM about once per step (halo rows and
// segment restarts come from L2); every new value is written once.
#include <cstring>

#include "step_common.cuh"
#include "step_launch.hpp"
#include "step_tiled.hpp"

namespace islbm {

namespace {

constexpr int NTHREADS = 256;
constexpr int NSTAGES = 4;

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
// to its end (no thread can be left behind at a barrier).
// After one timeout the thread stops waiting altogether (`faulted`), so a broken pipeline
// costs one bounded wait, not one per plane.
__device__ __forceinline__ void mbar_wait(uint64_t *bar, unsigned parity, Ctrl *ctrl, bool &faulted) {
    if (faulted) return;
    for (int it = 0; it < (1 << 22); ++it) {
        if (mbar_try_wait(bar, parity)) return;
        if (it > 32) __nanosleep(256);
    }
    faulted = true;
    atomicOr(&ctrl->fault, 1u);
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// four consecutive stored values -> float (deviation formats add the lattice weight)
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
__device__ __forceinline__ float4 ld4(const float *p) { return *(const float4 *)p; }

__device__ __forceinline__ int wrapi(int v, int n) {
    v %= n;
    return v < 0 ? v + n : v;
}

// BFL rows (C/evolution.h:505-572) for one node, reading the old populations from global
// memory; rare (flagged wall rows only), kept out of line.
template <class S>
__device__ __noinline__ void bfl_node(const S *__restrict__ fo, const Tables<float> &T, const StepConst &k, int x, int y, int z,
                                      float *F) {
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

struct Ring {
    // xi-ring of filtered values, slot k = plane (p - 6 + k); pairs of directions
    float2 r12[7], r34[7], r56[7], r78[7], r910[7], r1112[7], r1314[7], r1516[7], r1718[7];
    __device__ __forceinline__ void shift() {
#pragma unroll
        for (int s = 0; s < 6; s++) {
            r12[s] = r12[s + 1]; r34[s] = r34[s + 1]; r56[s] = r56[s + 1]; r78[s] = r78[s + 1]; r910[s] = r910[s + 1];
            r1112[s] = r1112[s + 1]; r1314[s] = r1314[s + 1]; r1516[s] = r1516[s + 1]; r1718[s] = r1718[s + 1];
        }
    }
};

template <class S, bool LES>
struct TiledKernel {
    // per-launch float constants (computed once per thread from the FP64 controller state)
    struct Scal { float f6, f12, rho_mod, tau, lesC; };
    const S *__restrict__ fo;
    S *__restrict__ fn;
    Tables<float> T;
    StepConst k;
    TiledConst tc;
    Ctrl *ctrl;
    float *rho_out, *u_out, *v_out, *w_out;
    int macros_on, mass_on;

    // one target node: xi combination, walls, BFL, collision, store. `wv` points at the 64 xi
    // weights of (y, z) (shared memory for interior targets, global for the wall caps).
    template <int SLOT12>
    __device__ __forceinline__ void target(const Ring &R, int x, int y, int z, const float *wv_, float f0, const Scal &sc,
                                           double &ub, double &mass) const {
        const int NX = k.NX, NY = k.NY;
        const size_t N = (size_t)NX*NY*k.NZ;
        const size_t node = ((size_t)z*NY + y)*NX + x;
        const float4 *wv = (const float4 *)wv_;
        float F[19];
        F[0] = f0;
        F[1] = R.r12[SLOT12].x; F[2] = R.r12[SLOT12].y;
        // xi combination, one weight table at a time (8 live weights instead of 56)
        auto table = [&](int t, float (&w)[7]) {
            const float4 a = wv[2*t], b = wv[2*t + 1];
            w[0] = a.x; w[1] = a.y; w[2] = a.z; w[3] = a.w; w[4] = b.x; w[5] = b.y; w[6] = b.z;
        };
        {
            float w[7];
            table(XI3, w);
            float f3 = 0, f7 = 0, f8 = 0;
#pragma unroll
            for (int c = 0; c < 7; c++) { f3 += w[c]*R.r34[c].x; f7 += w[c]*R.r78[c].x; f8 += w[c]*R.r78[c].y; }
            F[3] = f3; F[7] = f7; F[8] = f8;
            table(XI4, w);
            float f4 = 0, f9 = 0, f10 = 0;
#pragma unroll
            for (int c = 0; c < 7; c++) { f4 += w[c]*R.r34[c].y; f9 += w[c]*R.r910[c].x; f10 += w[c]*R.r910[c].y; }
            F[4] = f4; F[9] = f9; F[10] = f10;
            table(XI5, w);
            float f5 = 0, f11 = 0, f12 = 0;
#pragma unroll
            for (int c = 0; c < 7; c++) { f5 += w[c]*R.r56[c].x; f11 += w[c]*R.r1112[c].x; f12 += w[c]*R.r1112[c].y; }
            F[5] = f5; F[11] = f11; F[12] = f12;
            table(XI6, w);
            float f6 = 0, f13 = 0, f14 = 0;
#pragma unroll
            for (int c = 0; c < 7; c++) { f6 += w[c]*R.r56[c].y; f13 += w[c]*R.r1314[c].x; f14 += w[c]*R.r1314[c].y; }
            F[6] = f6; F[13] = f13; F[14] = f14;
            float g = 0;
            table(XI15, w);
#pragma unroll
            for (int c = 0; c < 7; c++) g += w[c]*R.r1516[c].x;
            F[15] = g; g = 0;
            table(XI16, w);
#pragma unroll
            for (int c = 0; c < 7; c++) g += w[c]*R.r1516[c].y;
            F[16] = g; g = 0;
            table(XI17, w);
#pragma unroll
            for (int c = 0; c < 7; c++) g += w[c]*R.r1718[c].x;
            F[17] = g; g = 0;
            table(XI18, w);
#pragma unroll
            for (int c = 0; c < 7; c++) g += w[c]*R.r1718[c].y;
            F[18] = g;
        }

        if (z == 0) {
            const S *b = fo + node;
            F[5] = load_f<S>(b + 6*N, 0, 6); F[11] = load_f<S>(b + 14*N, 0, 14); F[12] = load_f<S>(b + 13*N, 0, 13);
            F[15] = load_f<S>(b + 18*N, 0, 18); F[16] = load_f<S>(b + 17*N, 0, 17);
        }
        if (z == k.NZ - 1) {
            const S *b = fo + node;
            F[6] = load_f<S>(b + 5*N, 0, 5); F[13] = load_f<S>(b + 12*N, 0, 12); F[14] = load_f<S>(b + 11*N, 0, 11);
            F[17] = load_f<S>(b + 16*N, 0, 16); F[18] = load_f<S>(b + 15*N, 0, 15);
        }
        if (z <= 1) {
            const int nb = 2*k.NYD6, r = z*k.NYD6 + (y + 3);
            if (T.bfl_flag[r] | T.bfl_flag[nb + r] | T.bfl_flag[2*nb + r] | T.bfl_flag[3*nb + r]) bfl_node<S>(fo, T, k, x, y, z, F);
        }
        float rho_s, u1, v1, w1;
        collide_node<float, LES>(F, sc.rho_mod, sc.f6, sc.f12, sc.tau, sc.lesC, rho_s, u1, v1, w1);
#pragma unroll
        for (int q = 0; q < 19; q++) store_f<S>(fn + (size_t)q*N, node, q, F[q]);
        if (macros_on) { rho_out[node] = rho_s; u_out[node] = u1; v_out[node] = v1; w_out[node] = w1; }
        if (y == k.yplane) ub += (double)v1*T.dxv[x]*T.dzv[z];
        if (mass_on) mass += rho_s;
        if (!(rho_s == rho_s)) ctrl->nonfinite = 1u;
    }

    // Copies of plane p into one stage: the 18 moving populations (with the streamwise halo
    // where needed) and, when plane p completes the window of an interior target z = p - 3,
    // that target's xi weights and f0 row.
    // Issued by warp 0: lane 0 posts the expected bytes, then lane q copies population q
    // (two pieces when the halo wraps) and lanes 19, 20 the target data.
    __device__ void issue_plane(unsigned char *stage, uint64_t *bar, int p, int y0, int lane) const {
        const int NX = k.NX, NY = k.NY, NZ = k.NZ, TY = tc.TY;
        const size_t N = (size_t)NX*NY*NZ;
        const unsigned row_bytes = (unsigned)(NX*sizeof(S));
        const bool tgt = p >= 7 && p <= NZ - 1;
        if (lane == 0) mbar_expect_tx(bar, tc.stage_bytes_used + (tgt ? tc.tgt_bytes : 0u));
        __syncwarp();
        S *pops = (S *)stage;
        const int q = lane;
        if (q >= 1 && q < 19) {
            S *dst = pops + tc.off[q];
            const S *plane_base = fo + (size_t)q*N + (size_t)p*NY*NX;
            if (tc.rows[q] == TY) {
                bulk_g2s(dst, plane_base + (size_t)y0*NX, TY*row_bytes, bar);
            } else {
                const int ys = y0 >= 3 ? y0 - 3 : y0 - 3 + NY;
                const int rows = TY + 6;
                const int first = min(rows, NY - ys);
                bulk_g2s(dst, plane_base + (size_t)ys*NX, first*row_bytes, bar);
                if (first < rows) bulk_g2s(dst + (size_t)first*NX, plane_base, (rows - first)*row_bytes, bar);
            }
        }
        if (tgt && lane == 19) {
            const int z = p - 3;
            bulk_g2s(stage + tc.w_off, T.wxi + ((size_t)z*NY + y0)*64, (unsigned)(TY*64*sizeof(float)), bar);
        }
        if (tgt && lane == 20) {
            const int z = p - 3;
            bulk_g2s(stage + tc.f0_off, fo + ((size_t)z*NY + y0)*NX, TY*row_bytes, bar);
        }
    }

    struct Lane {
        int tid, xl, yl;        // node of this thread within the tile
        int xr, xx0;            // spanwise-filter task: row and first of two nodes
        int xsel;               // 0: departure x - minSize (7, 9, 1, 11, 13), 1: x + minSize
    };

    // One source plane: wait for its copies, advance the ring, filter, store into ring slot 6.
    __device__ __forceinline__ void plane(int i, int p, int p1, int y0, unsigned char *smem, Ring &R, unsigned &parity,
                                          bool &faulted, const Lane &L) const {
        const int NX = k.NX, TY = tc.TY;
        const int s = i % NSTAGES;
        uint64_t *bars = (uint64_t *)(smem + tc.bar_off);
        float *ybuf = (float *)(smem + tc.ybuf_off);   // [4][TY][NX]  dirs 7, 8, 9, 10
        float *xbuf = (float *)(smem + tc.xbuf_off);   // [10][TY][NX] dirs 7..10, 1, 2, 11..14
        unsigned char *stage = smem + (size_t)s*tc.stage_bytes;
        const S *raw = (const S *)stage;
        mbar_wait(&bars[s], (parity >> s) & 1u, ctrl, faulted);
        parity ^= 1u << s;
        R.shift();
        {   // streamwise filter over rows yl .. yl+6 of the halo copy, and raw values of 5, 6
            auto row = [&](int q, int lr) -> const S * { return raw + tc.off[q] + lr*NX + L.xl; };
            float a3 = 0, a4 = 0, a15 = 0, a16 = 0, a17 = 0, a18 = 0, a7 = 0, a8 = 0, a9 = 0, a10 = 0;
#pragma unroll
            for (int b = 0; b < 7; b++) {
                const float y0w = tc.wy0[b], y2w = tc.wy2[b];
                const int lr = L.yl + b;
                a3 += y0w*ld1<S>(row(3, lr), 1.f/18); a4 += y2w*ld1<S>(row(4, lr), 1.f/18);
                a15 += y0w*ld1<S>(row(15, lr), 1.f/36); a16 += y2w*ld1<S>(row(16, lr), 1.f/36);
                a17 += y0w*ld1<S>(row(17, lr), 1.f/36); a18 += y2w*ld1<S>(row(18, lr), 1.f/36);
                a7 += y0w*ld1<S>(row(7, lr), 1.f/36); a8 += y0w*ld1<S>(row(8, lr), 1.f/36);
                a9 += y2w*ld1<S>(row(9, lr), 1.f/36); a10 += y2w*ld1<S>(row(10, lr), 1.f/36);
            }
            R.r34[6] = make_float2(a3, a4);
            R.r1516[6] = make_float2(a15, a16);
            R.r1718[6] = make_float2(a17, a18);
            R.r56[6] = make_float2(ld1<S>(row(5, L.yl), 1.f/18), ld1<S>(row(6, L.yl), 1.f/18));
            const int o = L.yl*NX + L.xl;
            ybuf[0*TY*NX + o] = a7; ybuf[1*TY*NX + o] = a8; ybuf[2*TY*NX + o] = a9; ybuf[3*TY*NX + o] = a10;
        }
        __syncthreads();
        // every thread has finished plane i-1: its stage can take plane i + NSTAGES - 1
        if (L.tid < 32 && p + NSTAGES - 1 <= p1) {
            fence_proxy_async();
            const int sn = (i + NSTAGES - 1) % NSTAGES;
            issue_plane(smem + (size_t)sn*tc.stage_bytes, &bars[sn], p + NSTAGES - 1, y0, L.tid);
        }
        {   // spanwise filter: two nodes of one row, five directions of one departure side
            const int m = NX - 1;
            const int x0 = L.xx0;
            const int xa = (x0 - 4) & m, xb = (x0 - 2) & m, xc = x0, xd = (x0 + 2) & m, xe = (x0 + 4) & m;
#pragma unroll
            for (int j = 0; j < 5; j++) {
                const int d = 2*j + L.xsel;        // xbuf slot: 7, 8, 9, 10, 1, 2, 11, 12, 13, 14
                float v[10];
                if (j < 2) {
                    const float *in = ybuf + (size_t)d*TY*NX + L.xr*NX;
                    const float2 a = *(const float2 *)(in + xa), b = *(const float2 *)(in + xb), c = *(const float2 *)(in + xc),
                                 e = *(const float2 *)(in + xd), g = *(const float2 *)(in + xe);
                    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y; v[4] = c.x; v[5] = c.y; v[6] = e.x; v[7] = e.y; v[8] = g.x; v[9] = g.y;
                } else {
                    const int q = d == 4 ? 1 : (d == 5 ? 2 : d + 5);
                    const float w = q <= 2 ? 1.f/18 : 1.f/36;
                    const S *in = raw + tc.off[q] + L.xr*NX;
                    v[0] = ld1<S>(in + xa, w); v[1] = ld1<S>(in + xa + 1, w); v[2] = ld1<S>(in + xb, w); v[3] = ld1<S>(in + xb + 1, w);
                    v[4] = ld1<S>(in + xc, w); v[5] = ld1<S>(in + xc + 1, w); v[6] = ld1<S>(in + xd, w); v[7] = ld1<S>(in + xd + 1, w);
                    v[8] = ld1<S>(in + xe, w); v[9] = ld1<S>(in + xe + 1, w);
                }
                float o0 = 0, o1 = 0;
#pragma unroll
                for (int a = 0; a < 7; a++) {
                    const float w = L.xsel ? tc.wx2[a] : tc.wx0[a];
                    o0 += w*v[a + 1]; o1 += w*v[a + 2];
                }
                *(float2 *)(xbuf + (size_t)d*TY*NX + L.xr*NX + x0) = make_float2(o0, o1);
            }
        }
        __syncthreads();
        {
            const int o = L.yl*NX + L.xl, st = TY*NX;
            R.r78[6] = make_float2(xbuf[0*st + o], xbuf[1*st + o]);
            R.r910[6] = make_float2(xbuf[2*st + o], xbuf[3*st + o]);
            R.r12[6] = make_float2(xbuf[4*st + o], xbuf[5*st + o]);
            R.r1112[6] = make_float2(xbuf[6*st + o], xbuf[7*st + o]);
            R.r1314[6] = make_float2(xbuf[8*st + o], xbuf[9*st + o]);
        }
    }

    template <int SLOT12>
    __device__ __forceinline__ void cap_target(const Ring &R, int x, int y, int z, const Scal &sc, double &ub,
                                               double &mass) const {
        const size_t node = ((size_t)z*k.NY + y)*k.NX + x;
        target<SLOT12>(R, x, y, z, T.wxi + ((size_t)z*k.NY + y)*64, load_f<S>(fo, node, 0), sc, ub, mass);
    }

    __device__ void run() const {
        extern __shared__ __align__(128) unsigned char smem[];
        const int NX = k.NX, NZ = k.NZ, TY = tc.TY;
        uint64_t *bars = (uint64_t *)(smem + tc.bar_off);
        Lane L;
        L.tid = threadIdx.x;
        L.xl = L.tid & (NX - 1);
        L.yl = L.tid >> tc.log2nx;
        L.xsel = L.tid >> 7;                           // 128 threads per departure side
        const int pair = L.tid & 127;                  // TY*NX/2 = 128 node pairs per plane
        L.xr = pair >> (tc.log2nx - 1);
        L.xx0 = 2*(pair & (NX/2 - 1));

        if (L.tid == 0) {
            for (int s = 0; s < NSTAGES; s++) mbar_init(&bars[s], 1);
            fence_mbar_init();
        }
        __syncthreads();
        unsigned parity = 0;   // bit s: parity of the next completion of stage s
        bool faulted = false;

        double ub = 0.0, mass = 0.0;
        Scal sc;
        {
            const double force = ctrl->force;
            sc.f6 = (float)(1.0/6*force*k.dt);
            sc.f12 = (float)(1.0/12*force*k.dt);
            sc.rho_mod = (float)ctrl->rho_modify;
            sc.tau = (float)k.tau;
            sc.lesC = (float)k.les_C;
        }
        Ring R;
#pragma unroll
        for (int s = 0; s < 7; s++) {
            R.r12[s] = R.r34[s] = R.r56[s] = R.r78[s] = R.r910[s] = make_float2(0.f, 0.f);
            R.r1112[s] = R.r1314[s] = R.r1516[s] = R.r1718[s] = make_float2(0.f, 0.f);
        }
        // whole columns: CTA b takes tiles b, b + G, b + 2G, ... so that the CTAs running at the
        // same time hold neighbouring tiles at similar heights and share the halo rows in L2
        const int ntiles = k.NY/TY;
        for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
            const int za = 0, zb = NZ;
            const int y0 = tile*TY;
            const int zl = zb - 1;
            const int p0 = za <= 3 ? 0 : (za >= NZ - 3 ? NZ - 7 : za - 3);
            const int p1 = zl <= 3 ? 6 : (zl >= NZ - 4 ? NZ - 1 : zl + 3);
            __syncthreads();   // every thread is done with every stage of the previous segment
            if (L.tid < 32) {
                fence_proxy_async();
                for (int s = 0; s < NSTAGES - 1 && p0 + s <= p1; s++)
                    issue_plane(smem + (size_t)s*tc.stage_bytes, &bars[s], p0 + s, y0, L.tid);
            }
            const int y = y0 + L.yl;
            int i = 0, p = p0;
            // warm-up: the six planes below the first window end
#pragma unroll 1
            for (; i < 6; i++, p++) plane(i, p, p1, y0, smem, R, parity, faulted, L);
            if (p == 6) {   // window of the lower wall cap (targets 0..3 share planes 0..6)
                plane(i, p, p1, y0, smem, R, parity, faulted, L);
                if (za <= 0 && 0 < zb) cap_target<0>(R, L.xl, y, 0, sc, ub, mass);
                if (za <= 1 && 1 < zb) cap_target<1>(R, L.xl, y, 1, sc, ub, mass);
                if (za <= 2 && 2 < zb) cap_target<2>(R, L.xl, y, 2, sc, ub, mass);
                if (za <= 3 && 3 < zb) cap_target<3>(R, L.xl, y, 3, sc, ub, mass);
                i++; p++;
            }
            // steady state: each plane completes the window of one interior target
            const int pend = min(p1, NZ - 2);
#pragma unroll 1
            for (; p <= pend; i++, p++) {
                plane(i, p, p1, y0, smem, R, parity, faulted, L);
                const unsigned char *stage = smem + (size_t)(i % NSTAGES)*tc.stage_bytes;
                const float *wv = (const float *)(stage + tc.w_off) + L.yl*64;
                const float f0 = ld1<S>((const S *)(stage + tc.f0_off) + L.yl*NX + L.xl, 1.f/3);
                target<3>(R, L.xl, y, p - 3, wv, f0, sc, ub, mass);
            }
            if (p == NZ - 1 && p <= p1) {   // window of the upper wall cap
                plane(i, p, p1, y0, smem, R, parity, faulted, L);
                const int zt = NZ - 4;
                if (za <= zt && zt < zb) {
                    const unsigned char *stage = smem + (size_t)(i % NSTAGES)*tc.stage_bytes;
                    const float *wv = (const float *)(stage + tc.w_off) + L.yl*64;
                    const float f0 = ld1<S>((const S *)(stage + tc.f0_off) + L.yl*NX + L.xl, 1.f/3);
                    target<3>(R, L.xl, y, zt, wv, f0, sc, ub, mass);
                }
                if (za <= NZ - 3 && NZ - 3 < zb) cap_target<4>(R, L.xl, y, NZ - 3, sc, ub, mass);
                if (za <= NZ - 2 && NZ - 2 < zb) cap_target<5>(R, L.xl, y, NZ - 2, sc, ub, mass);
                if (za <= NZ - 1 && NZ - 1 < zb) cap_target<6>(R, L.xl, y, NZ - 1, sc, ub, mass);
            }
        }
        end_of_step<NTHREADS>(ctrl, k, tc.n, ub, mass, true, mass_on != 0);
    }
};

template <class S, bool LES>
__global__ void __launch_bounds__(NTHREADS, 1) step_tiled_kernel(TiledKernel<S, LES> K) { K.run(); }

template <class S, bool LES>
cudaError_t launch_t(const StepLaunch &L) {
    TiledKernel<S, LES> K;
    K.fo = (const S *)L.fo;
    K.fn = (S *)L.fn;
    K.T = *(const Tables<float> *)L.tables;
    K.k = L.k;
    K.tc = *(const TiledConst *)L.tiled;
    K.tc.n = L.n;
    K.ctrl = L.ctrl;
    K.rho_out = (float *)L.macros[0]; K.u_out = (float *)L.macros[1];
    K.v_out = (float *)L.macros[2]; K.w_out = (float *)L.macros[3];
    K.macros_on = L.macros_on; K.mass_on = L.mass;
    static size_t attr_smem = 0;   // largest dynamic shared memory enabled for this instantiation
    const size_t smem = K.tc.smem_bytes;
    if (smem > attr_smem) {
        cudaError_t e = cudaFuncSetAttribute(step_tiled_kernel<S, LES>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr_smem = smem;
    }
    step_tiled_kernel<S, LES><<<K.tc.grid, NTHREADS, smem, L.stream>>>(K);
    return cudaGetLastError();
}

template <class S>
cudaError_t launch_s(const StepLaunch &L) {
    return L.les ? launch_t<S, true>(L) : launch_t<S, false>(L);
}

size_t elem_bytes(int precision) { return precision == ISLBM_FP32 ? 4 : 2; }

}  // namespace

bool tiled_supported(const StepConst &k, int precision) {
    if (precision == ISLBM_FP64) return false;
    // NX a power of two in [8, 256] so that a tile is 256 nodes and index math is shifts
    if (k.NX < 8 || k.NX > NTHREADS || (k.NX & (k.NX - 1)) != 0) return false;
    const int TY = NTHREADS/k.NX;
    if (k.NY % TY != 0 || k.NY < TY + 6 || k.NZ < 8) return false;
    return true;
}

int make_tiled_const(const StepConst &k, int precision, const double *wx0, const double *wx2, const double *wy0,
                     const double *wy2, int num_sms, TiledConst *out) {
    TiledConst tc;
    std::memset(&tc, 0, sizeof(tc));
    tc.TY = NTHREADS/k.NX;
    int l = 0;
    while ((1 << l) < k.NX) l++;
    tc.log2nx = l;
    const size_t eb = elem_bytes(precision);
    auto up16 = [](size_t v) { return (v + 15)/16*16; };
    size_t off = 0;   // bytes within a stage
    tc.off[0] = 0; tc.rows[0] = 0;
    size_t used = 0;
    for (int q = 1; q < 19; q++) {
        const bool wide = (q == 3 || q == 4 || (q >= 7 && q <= 10) || q >= 15);
        tc.rows[q] = wide ? tc.TY + 6 : tc.TY;
        tc.off[q] = (int)(off/eb);
        off = up16(off + (size_t)tc.rows[q]*k.NX*eb);
        used += (size_t)tc.rows[q]*k.NX*eb;
    }
    tc.stage_bytes_used = (unsigned)used;
    tc.w_off = (unsigned)off;
    off = up16(off + (size_t)tc.TY*64*sizeof(float));
    tc.f0_off = (unsigned)off;
    off = up16(off + (size_t)tc.TY*k.NX*eb);
    tc.tgt_bytes = (unsigned)(tc.TY*64*sizeof(float) + tc.TY*k.NX*eb);
    tc.stage_bytes = (off + 127)/128*128;
    tc.ybuf_off = NSTAGES*tc.stage_bytes;
    tc.xbuf_off = tc.ybuf_off + (size_t)4*tc.TY*k.NX*sizeof(float);
    tc.bar_off = tc.xbuf_off + (size_t)10*tc.TY*k.NX*sizeof(float);
    tc.smem_bytes = tc.bar_off + NSTAGES*sizeof(uint64_t);
    for (int a = 0; a < 7; a++) {
        tc.wx0[a] = (float)wx0[a]; tc.wx2[a] = (float)wx2[a];
        tc.wy0[a] = (float)wy0[a]; tc.wy2[a] = (float)wy2[a];
    }
    const int tiles = k.NY/tc.TY;
    tc.units = (long long)tiles*k.NZ;
    tc.grid = tiles < num_sms ? tiles : num_sms;
    *out = tc;
    return tc.smem_bytes <= 227*1024 ? 0 : -1;
}

cudaError_t launch_step_tiled(const StepLaunch &L) {
    switch (L.precision) {
    case ISLBM_FP32: return launch_s<float>(L);
    case ISLBM_FP16_DEV: return launch_s<__half>(L);
    case ISLBM_BF16_DEV: return launch_s<__nv_bfloat16>(L);
    default: return cudaErrorNotSupported;
    }
}

}  // namespace islbm
