// Tiled step kernel: z-marching x-y tiles staged in shared memory by bulk async copies.
//
// Same step as stream_collide (C/evolution.h:358-684) for FP32 arithmetic with FP32, FP16 or
// BF16 population storage, organised for HBM:
//   * a CTA owns a tile of TY = 128/NX full-width rows (all NX spanwise nodes) and marches
//     upward through the wall-normal planes of that column; every plane of the 18 moving
//     populations is copied global -> shared with cp.async.bulk (one copy per population and
//     plane, 3-row streamwise halo for the ten populations with e_y != 0, periodic wrap by
//     splitting the copy), tracked by an mbarrier, 2 stages deep; the target plane's xi
//     weights and f0 row ride in the same stage;
//   * the interpolation is applied as separable filters, exact in real arithmetic because the
//     x and y weights are the same for every node (uniform spacing, C/initialization.h:51-108)
//     and the xi weights depend only on the target (y, z): a streamwise filter over the halo
//     rows, then a spanwise filter (2 nodes per task) through shared memory, then the xi
//     combination over a 7-plane ring of filtered values kept in registers (packed FP32x2
//     FMAs), so each loaded value feeds 7 target planes without being re-read;
//   * the collision tail, wall bounce-back, BFL rows and controller partial sums are fused;
//   * CTAs are persistent (2 per SM, 128 threads each) and take whole columns: CTA b takes
//     tiles b, b + G, b + 2G, ..., so CTAs running at the same time hold neighbouring tiles at
//     similar heights and share the streamwise halo rows through L2.
// Every value of the old populations is read from HBM about once per step (halo rows come
// from L2); every new value is written once.
#include <cstring>
#include <type_traits>

#include "step_common.cuh"
#include "step_launch.hpp"
#include "step_tiled.hpp"
#include "tile_helpers.cuh"

namespace islbm {

namespace {

constexpr int NTHREADS = 128;
// Copy stages per tile: the next plane is in flight while one is filtered (a third stage for
// the 2-byte formats, which would fit, measured no faster on GB300).
template <class S> constexpr int stages_for() { return 2; }

// Shared-memory layout of one tile for a spanwise width NXC (a power of two): all offsets are
// compile-time constants so every shared-memory address is a base plus an immediate.
//   stage s (NS of them): population q in [1, 18] as `rows(q)` rows of NXC values
//   (TY rows, or TY + 6 with the streamwise halo), then the target's xi weights (TY x 64
//   floats) and f0 row (TY x NXC values); then ybuf [4][TY][NXC] and xbuf [10][TY][NXC] floats,
//   then the stage mbarriers.
template <class S, int NXC>
struct Lay {
    static constexpr int NX = NXC;
    static constexpr int TY = NTHREADS/NXC;
    static constexpr int LOG2NX = NXC == 8 ? 3 : NXC == 16 ? 4 : NXC == 32 ? 5 : NXC == 64 ? 6 : NXC == 128 ? 7 : 8;
    static constexpr int EB = (int)sizeof(S);
    static constexpr int NS = stages_for<S>();
    static constexpr bool wide(int q) { return q == 3 || q == 4 || (q >= 7 && q <= 10) || q >= 15; }
    static constexpr int rows(int q) { return q == 0 ? 0 : (wide(q) ? TY + 6 : TY); }
    static constexpr int up16(int v) { return (v + 15)/16*16; }
    static constexpr int off_bytes(int q) {
        int off = 0;
        for (int r = 1; r < q; ++r) off = up16(off + rows(r)*NX*EB);
        return off;
    }
    static constexpr int off(int q) { return off_bytes(q)/EB; }
    static constexpr unsigned pops_bytes() {
        unsigned b = 0;
        for (int q = 1; q < 19; ++q) b += (unsigned)(rows(q)*NX*EB);
        return b;
    }
    static constexpr int w_off = off_bytes(19);
    static constexpr int f0_off = up16(w_off + TY*64*4);
    static constexpr int stage_bytes = (up16(f0_off + TY*NX*EB) + 127)/128*128;
    static constexpr unsigned tgt_bytes = (unsigned)(TY*64*4 + TY*NX*EB);
    static constexpr int ybuf_off = NS*stage_bytes;
    static constexpr int xbuf_off = ybuf_off + 4*TY*NX*4;
    static constexpr int bar_off = xbuf_off + 10*TY*NX*4;
    static constexpr int flag_off = bar_off + NS*8;   // CTA-wide "a wait timed out" flag
    static constexpr int smem_bytes = flag_off + 16;
};

// Filtered values of one plane for the node of this thread (pairs of directions).
struct Slot {
    float2 r12, r34, r56, r78, r910, r1112, r1314, r1516, r1718;
};

// xi ring: the 7 planes of the current window in registers, slot (p mod 7) holding plane p.
// Slot indices are compile-time constants in every access (the 7 window phases are
// instantiated separately), so the ring is never shifted.
struct Ring {
    Slot s[7];
};

// xi combination of the window whose newest plane sits in slot NEW (oldest in NEW + 1).
// The 64 weights of (y, z) are interleaved per stencil point c: (xi3, xi4, xi5, xi6, xi15,
// xi16, xi17, xi18)[c], so one float4 yields the weight pairs of the packed FMAs.
// Returns F[3..18] and F1, F2 of the plane three below the newest one.
template <int NEW>
__device__ __forceinline__ void xi_combine(const Ring &R, const float *wv_, float *F) {
    const float4 *wv = (const float4 *)wv_;
    constexpr int O = (NEW + 1) % 7;   // slot of the oldest plane (c = 0)
    P2 a34 = p2(0.f, 0.f), a56 = a34, a1516 = a34, a1718 = a34, a78 = a34, a910 = a34, a1112 = a34, a1314 = a34;
#pragma unroll
    for (int c = 0; c < 7; c++) {
        const Slot &q = R.s[(O + c) % 7];
        const float4 w = wv[2*c], u = wv[2*c + 1];
        fma2(a34, p2(w.x, w.y), p2(q.r34));
        fma2(a56, p2(w.z, w.w), p2(q.r56));
        fma2(a1516, p2(u.x, u.y), p2(q.r1516));
        fma2(a1718, p2(u.z, u.w), p2(q.r1718));
        fma2(a78, p2(w.x, w.x), p2(q.r78));
        fma2(a910, p2(w.y, w.y), p2(q.r910));
        fma2(a1112, p2(w.z, w.z), p2(q.r1112));
        fma2(a1314, p2(w.w, w.w), p2(q.r1314));
    }
    constexpr int MID = (NEW + 4) % 7;   // plane p - 3
    F[1] = R.s[MID].r12.x; F[2] = R.s[MID].r12.y;
    float2 t;
    t = unp(a34); F[3] = t.x; F[4] = t.y;
    t = unp(a56); F[5] = t.x; F[6] = t.y;
    t = unp(a78); F[7] = t.x; F[8] = t.y;
    t = unp(a910); F[9] = t.x; F[10] = t.y;
    t = unp(a1112); F[11] = t.x; F[12] = t.y;
    t = unp(a1314); F[13] = t.x; F[14] = t.y;
    t = unp(a1516); F[15] = t.x; F[16] = t.y;
    t = unp(a1718); F[17] = t.x; F[18] = t.y;
}

// the window phase selects the instantiation
__device__ __forceinline__ void xi_combine_phase(int ph, const Ring &R, const float *wv, float *F) {
    switch (ph) {
    case 0: xi_combine<0>(R, wv, F); break;
    case 1: xi_combine<1>(R, wv, F); break;
    case 2: xi_combine<2>(R, wv, F); break;
    case 3: xi_combine<3>(R, wv, F); break;
    case 4: xi_combine<4>(R, wv, F); break;
    case 5: xi_combine<5>(R, wv, F); break;
    default: xi_combine<6>(R, wv, F); break;
    }
}

__device__ __forceinline__ void ring_store(Ring &R, int ph, const Slot &v) {
    switch (ph) {
    case 0: R.s[0] = v; break;
    case 1: R.s[1] = v; break;
    case 2: R.s[2] = v; break;
    case 3: R.s[3] = v; break;
    case 4: R.s[4] = v; break;
    case 5: R.s[5] = v; break;
    default: R.s[6] = v; break;
    }
}

template <class S, bool LES, int NXC>
struct TiledKernel {
    using LY = Lay<S, NXC>;
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

    // Walls, BFL rows, collision and store of one node whose streamed populations are in F
    // (F[1..18] as filtered values, deviations for the deviation formats; F[0] full).
    __device__ __forceinline__ void finish(float *F, int x, int y, int z, const Scal &sc, float &ub, float &mass) const {
        constexpr int NX = LY::NX;
        const int NY = k.NY;
        const size_t N = (size_t)NX*NY*k.NZ;
        const size_t node = ((size_t)z*NY + y)*NX + x;
        if constexpr (Storage<S>::dev) {
#pragma unroll
            for (int q = 1; q < 19; q++) F[q] += (float)dev_ref(q);
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
        float Fl[19];
#pragma unroll
        for (int q = 0; q < 19; q++) Fl[q] = F[q];
        float rho_s, u1, v1, w1;
        collide_node<float, LES>(Fl, sc.rho_mod, sc.f6, sc.f12, sc.tau, sc.lesC, rho_s, u1, v1, w1);
#pragma unroll
        for (int q = 0; q < 19; q++) store_f<S>(fn + (size_t)q*N, node, q, Fl[q]);
        if (macros_on) { rho_out[node] = rho_s; u_out[node] = u1; v_out[node] = v1; w_out[node] = w1; }
        // column partials in FP32 (at most NZ terms), folded into FP64 once per column
        if (y == k.yplane) ub += v1*T.dxf[x]*T.dzf[z];
        mass += rho_s;
        if (!(rho_s == rho_s)) ctrl->nonfinite = 1u;
    }

    // F1, F2 of a wall-cap target by direct spanwise gathers (the ring keeps only the plane
    // three below the newest one)
    __device__ __forceinline__ void cap_f12(int x, int y, int z, float *F) const {
        constexpr int NX = LY::NX;
        const int NY = k.NY;
        const size_t N = (size_t)NX*NY*k.NZ;
        const S *r1 = fo + 1*N + ((size_t)z*NY + y)*NX, *r2 = fo + 2*N + ((size_t)z*NY + y)*NX;
        float a = 0, b = 0;
#pragma unroll
        for (int t = 0; t < 7; t++) {
            const int xx = (x - 3 + t) & (NX - 1);
            a += tc.wx0[t]*ldv<S>(r1 + xx);
            b += tc.wx2[t]*ldv<S>(r2 + xx);
        }
        F[1] = a; F[2] = b;
    }

    // Copy job q of a plane (1..18: population q, two pieces when the halo wraps; 19, 20: the
    // target's xi weights and f0 row). Jobs are spread over the four warps (job q on warp q & 3,
    // lane q >> 2) so that no warp serialises all the copy issues; thread 0 posts the expected
    // bytes (a copy may complete before that: the phase cannot end while the arrival is due).
    __device__ void issue_plane(unsigned char *stage, uint64_t *bar, int p, int y0, int tid) const {
        constexpr int NX = LY::NX, TY = LY::TY;
        const int NY = k.NY, NZ = k.NZ;
        const size_t N = (size_t)NX*NY*NZ;
        const unsigned row_bytes = (unsigned)(NX*sizeof(S));
        const bool tgt = p >= 7 && p <= NZ - 1;
        if (tid == 0) mbar_expect_tx(bar, LY::pops_bytes() + (tgt ? LY::tgt_bytes : 0u));
        S *pops = (S *)stage;
        const int q = 4*(tid & 31) + (tid >> 5);   // lanes 0..5 only
        if (q >= 1 && q < 19) {
            S *dst = pops + LY::off(q);
            const S *plane_base = fo + (size_t)q*N + (size_t)p*NY*NX;
            if (!LY::wide(q)) {
                bulk_g2s(dst, plane_base + (size_t)y0*NX, TY*row_bytes, bar);
            } else {
                const int ys = y0 >= 3 ? y0 - 3 : y0 - 3 + NY;
                const int rows = TY + 6;
                const int first = min(rows, NY - ys);
                bulk_g2s(dst, plane_base + (size_t)ys*NX, first*row_bytes, bar);
                if (first < rows) bulk_g2s(dst + (size_t)first*NX, plane_base, (rows - first)*row_bytes, bar);
            }
        }
        if (tgt && q == 19) {
            const int z = p - 3;
            bulk_g2s(stage + LY::w_off, T.wxi + ((size_t)z*NY + y0)*64, (unsigned)(TY*64*sizeof(float)), bar);
        }
        if (tgt && q == 20) {
            const int z = p - 3;
            bulk_g2s(stage + LY::f0_off, fo + ((size_t)z*NY + y0)*NX, TY*row_bytes, bar);
        }
    }

    // Thread 0, at the end of the kernel: bounded wait for copies still pending (only after a
    // timeout; in a healthy run every copy has been consumed).
    __device__ __forceinline__ void drain(unsigned char *smem, unsigned parity, int tid) const {
        if (tid != 0) return;
        uint64_t *bars = (uint64_t *)(smem + LY::bar_off);
        for (int s = 0; s < LY::NS; s++) {
            if (!((parity >> (PEND + s)) & 1u)) continue;
            const unsigned ph = (parity >> (PPAR + s)) & 1u;
            for (int it = 0; it < (1 << 22); ++it) {
                if (mbar_try_wait(&bars[s], ph)) break;
                if (it > 32) __nanosleep(256);
            }
        }
    }

    struct Lane {
        int tid, xl, yl;        // node of this thread within the tile
        int xr, xx0;            // spanwise-filter task: row and first of two nodes
        int xsel;               // 0: departure x - minSize (7, 9, 1, 11, 13), 1: x + minSize
    };

    // After a CTA barrier, lanes 0..5 of every warp start the copies of plane p into stage s;
    // thread 0 (which posts the expected bytes) records the stage as pending. After a timed-out
    // wait anywhere in the CTA (the shared flag, written before the barrier) no copy starts.
    __device__ __forceinline__ void issue(unsigned char *smem, int s, int p, int y0, const Lane &L, unsigned &parity) const {
        if ((L.tid & 31) >= 6) return;
        if (*(volatile int *)(smem + LY::flag_off)) return;
        if (p == k.drill_plane) return;   // failure drill: this plane's copies never start
        fence_proxy_async();
        issue_plane(smem + (size_t)s*LY::stage_bytes, (uint64_t *)(smem + LY::bar_off) + s, p, y0, L.tid);
        if (L.tid == 0)
            parity = (parity & ~(1u << (PPAR + s))) | (((parity >> s) & 1u) << (PPAR + s)) | (1u << (PEND + s));
    }

    // One source plane: wait for its copies, filter, return the plane's slot values.
    __device__ __forceinline__ Slot plane(int i, int p, int p1, int y0, unsigned char *smem, unsigned &parity, bool &faulted,
                                          const Lane &L) const {
        constexpr int NX = LY::NX, TY = LY::TY;
        const int s = i % LY::NS;
        uint64_t *bars = (uint64_t *)(smem + LY::bar_off);
        float *ybuf = (float *)(smem + LY::ybuf_off);   // [4][TY][NX]  dirs 7, 8, 9, 10
        float *xbuf = (float *)(smem + LY::xbuf_off);   // [10][TY][NX] dirs 7..10, 1, 2, 11..14
        unsigned char *stage = smem + (size_t)s*LY::stage_bytes;
        const S *raw = (const S *)stage;
        if (mbar_wait(&bars[s], (parity >> s) & 1u, ctrl, faulted)) parity &= ~(1u << (PEND + s));
        else if (faulted) *(volatile int *)(smem + LY::flag_off) = 1;
        parity ^= 1u << s;
        Slot v;
        {   // streamwise filter over rows yl .. yl+6 of the halo copy, and raw values of 5, 6
            const S *base = raw + L.yl*NX + L.xl;
            auto row = [&](int q, int b) -> const S * { return base + LY::off(q) + b*NX; };
            float a3 = 0, a4 = 0, a15 = 0, a16 = 0, a17 = 0, a18 = 0, a7 = 0, a8 = 0, a9 = 0, a10 = 0;
#pragma unroll
            for (int b = 0; b < 7; b++) {
                const float y0w = tc.wy0[b], y2w = tc.wy2[b];
                a3 += y0w*ldv<S>(row(3, b)); a4 += y2w*ldv<S>(row(4, b));
                a15 += y0w*ldv<S>(row(15, b)); a16 += y2w*ldv<S>(row(16, b));
                a17 += y0w*ldv<S>(row(17, b)); a18 += y2w*ldv<S>(row(18, b));
                a7 += y0w*ldv<S>(row(7, b)); a8 += y0w*ldv<S>(row(8, b));
                a9 += y2w*ldv<S>(row(9, b)); a10 += y2w*ldv<S>(row(10, b));
            }
            v.r34 = make_float2(a3, a4);
            v.r1516 = make_float2(a15, a16);
            v.r1718 = make_float2(a17, a18);
            v.r56 = make_float2(ldv<S>(row(5, 0)), ldv<S>(row(6, 0)));
            const int o = L.yl*NX + L.xl;
            ybuf[0*TY*NX + o] = a7; ybuf[1*TY*NX + o] = a8; ybuf[2*TY*NX + o] = a9; ybuf[3*TY*NX + o] = a10;
        }
        __syncthreads();
        // every thread has finished plane i-1: its stage can take plane i + NS - 1
        if (p + LY::NS - 1 <= p1) issue(smem, (i + LY::NS - 1) % LY::NS, p + LY::NS - 1, y0, L, parity);
        {   // spanwise filter: two nodes of one row, five directions of one departure side
            const int m = NX - 1;
            const int x0 = L.xx0;
            const int xa = (x0 - 4) & m, xb = (x0 - 2) & m, xc = x0, xd = (x0 + 2) & m, xe = (x0 + 4) & m;
            auto task = [&](auto jc) {
                constexpr int j = decltype(jc)::value;
                const int d = 2*j + L.xsel;        // xbuf slot: 7, 8, 9, 10, 1, 2, 11, 12, 13, 14
                float vv[10];
                if constexpr (j < 2) {
                    const float *in = ybuf + (size_t)d*TY*NX + L.xr*NX;
                    const float2 a = *(const float2 *)(in + xa), b = *(const float2 *)(in + xb), c = *(const float2 *)(in + xc),
                                 e = *(const float2 *)(in + xd), g = *(const float2 *)(in + xe);
                    vv[0] = a.x; vv[1] = a.y; vv[2] = b.x; vv[3] = b.y; vv[4] = c.x; vv[5] = c.y; vv[6] = e.x; vv[7] = e.y; vv[8] = g.x; vv[9] = g.y;
                } else {
                    // population of this task: 1, 11, 13 (xsel 0) or 2, 12, 14 (xsel 1)
                    constexpr int qa = j == 2 ? 1 : (j == 3 ? 11 : 13);
                    constexpr int qb = j == 2 ? 2 : (j == 3 ? 12 : 14);
                    const S *in = raw + (L.xsel ? LY::off(qb) : LY::off(qa)) + L.xr*NX;
                    const float2 a = ldv2<S>(in + xa), b = ldv2<S>(in + xb), c = ldv2<S>(in + xc), e = ldv2<S>(in + xd),
                                 g = ldv2<S>(in + xe);
                    vv[0] = a.x; vv[1] = a.y; vv[2] = b.x; vv[3] = b.y; vv[4] = c.x; vv[5] = c.y; vv[6] = e.x; vv[7] = e.y; vv[8] = g.x; vv[9] = g.y;
                }
                float o0 = 0, o1 = 0;
#pragma unroll
                for (int a = 0; a < 7; a++) {
                    const float w = L.xsel ? tc.wx2[a] : tc.wx0[a];
                    o0 += w*vv[a + 1]; o1 += w*vv[a + 2];
                }
                *(float2 *)(xbuf + (size_t)d*TY*NX + L.xr*NX + x0) = make_float2(o0, o1);
            };
            task(std::integral_constant<int, 0>{}); task(std::integral_constant<int, 1>{});
            task(std::integral_constant<int, 2>{}); task(std::integral_constant<int, 3>{});
            task(std::integral_constant<int, 4>{});
        }
        __syncthreads();
        {
            const int o = L.yl*NX + L.xl, st = TY*NX;
            v.r78 = make_float2(xbuf[0*st + o], xbuf[1*st + o]);
            v.r910 = make_float2(xbuf[2*st + o], xbuf[3*st + o]);
            v.r12 = make_float2(xbuf[4*st + o], xbuf[5*st + o]);
            v.r1112 = make_float2(xbuf[6*st + o], xbuf[7*st + o]);
            v.r1314 = make_float2(xbuf[8*st + o], xbuf[9*st + o]);
        }
        return v;
    }

    // a wall-cap target: xi weights and f0 from global memory, F1/F2 by direct gathers
    __device__ __forceinline__ void cap_target(const Ring &R, int ph, int x, int y, int z, const Scal &sc, float &ub,
                                               float &mass) const {
        const size_t node = ((size_t)z*k.NY + y)*k.NX + x;
        float F[19];
        xi_combine_phase(ph, R, T.wxi + ((size_t)z*k.NY + y)*64, F);
        cap_f12(x, y, z, F);
        F[0] = load_f<S>(fo, node, 0);
        finish(F, x, y, z, sc, ub, mass);
    }

    __device__ __forceinline__ Lane lane() const {
        constexpr int NX = LY::NX;
        Lane L;
        L.tid = threadIdx.x;
        L.xl = L.tid & (NX - 1);
        L.yl = L.tid >> LY::LOG2NX;
        L.xsel = L.tid/(NTHREADS/2);                   // half the threads per departure side
        const int pair = L.tid & (NTHREADS/2 - 1);     // TY*NX/2 node pairs per plane
        L.xr = pair >> (LY::LOG2NX - 1);
        L.xx0 = 2*(pair & (NX/2 - 1));
        return L;
    }

    __device__ __forceinline__ Scal scalars() const {
        Scal sc;
        const double force = ctrl->force;
        sc.f6 = (float)(1.0/6*force*k.dt);
        sc.f12 = (float)(1.0/12*force*k.dt);
        sc.rho_mod = (float)ctrl->rho_modify;
        sc.tau = (float)k.tau;
        sc.lesC = (float)k.les_C;
        return sc;
    }

    // One whole column (tile rows y0 .. y0+TY-1, all planes): returns its partial sums.
    __device__ __forceinline__ void column(int tile, unsigned char *smem, Ring &R, unsigned &parity, bool &faulted,
                                           const Lane &L, const Scal &sc, float &ub, float &mass) const {
        constexpr int NX = LY::NX, TY = LY::TY;
        const int NZ = k.NZ;
        uint64_t *bars = (uint64_t *)(smem + LY::bar_off);
        const int y0 = tile*TY;
        const int p1 = NZ - 1;
        __syncthreads();   // every thread is done with every stage of the previous column
        for (int s = 0; s < LY::NS - 1 && s <= p1; s++) issue(smem, s, s, y0, L, parity);
        const int y = y0 + L.yl;
        // planes 0..6 fill the ring (plane p in slot p mod 7); then the lower cap
#pragma unroll 1
        for (int p = 0; p < 7; p++) {
            const Slot v = plane(p, p, p1, y0, smem, parity, faulted, L);
            ring_store(R, p, v);
        }
        for (int zt = 0; zt < 4; zt++) cap_target(R, 6, L.xl, y, zt, sc, ub, mass);
        // steady state: each plane completes the window of one interior target
        int ph = 0;   // slot of the newest plane = p mod 7
#pragma unroll 1
        for (int p = 7; p <= NZ - 1; p++) {
            const Slot v = plane(p, p, p1, y0, smem, parity, faulted, L);
            ring_store(R, ph, v);
            const unsigned char *stage = smem + (size_t)(p % LY::NS)*LY::stage_bytes;
            const float *wv = (const float *)(stage + LY::w_off) + L.yl*64;
            float F[19];
            xi_combine_phase(ph, R, wv, F);
            F[0] = ld1<S>((const S *)(stage + LY::f0_off) + L.yl*NX + L.xl, (float)dev_ref(0));
            finish(F, L.xl, y, p - 3, sc, ub, mass);
            ph = ph == 6 ? 0 : ph + 1;
        }
        // upper cap: targets NZ-3 .. NZ-1 share the last window (newest plane NZ-1)
        const int phl = (NZ - 1) % 7;
        for (int zt = NZ - 3; zt < NZ; zt++) cap_target(R, phl, L.xl, y, zt, sc, ub, mass);
    }

    __device__ void run() const {
        extern __shared__ __align__(128) unsigned char smem[];
        uint64_t *bars = (uint64_t *)(smem + LY::bar_off);
        const Lane L = lane();
        if (L.tid == 0) {
            for (int s = 0; s < LY::NS; s++) mbar_init(&bars[s], 1);
            *(volatile int *)(smem + LY::flag_off) = 0;
            fence_mbar_init();
        }
        __syncthreads();
        unsigned parity = 0;   // bit s: parity of the next completion of stage s
        bool faulted = false;
        double ub_total = 0.0, mass_total = 0.0;
        const Scal sc = scalars();
        Ring R;
        // whole columns: CTA b takes tiles b, b + G, b + 2G, ... so that the CTAs running at the
        // same time hold neighbouring tiles at similar heights and share the halo rows in L2
        const int ntiles = k.NY/LY::TY;
        for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
            float ub = 0.f, mass = 0.f;   // this column's partial sums
            column(tile, smem, R, parity, faulted, L, sc, ub, mass);
            ub_total += (double)ub;
            mass_total += (double)mass;
        }
        drain(smem, parity, L.tid);
        end_of_step<NTHREADS>(ctrl, k, tc.n, ub_total, mass_total, true, mass_on != 0,
                              gridDim.x*gridDim.y*gridDim.z);
    }
};

// Batched form: one launch advances every solve of a batch (same storage format and spanwise
// width) by one step. Work items are (solve, tile) pairs; a CTA copies the solve's
// descriptor into shared memory, takes the old/new buffers from the solve's own step
// counter (so a graph of identical launches advances the solves step after step), runs the
// column and reports it to the solve's controller, whose last column closes the step.
template <class S, bool LES, int NXC>
struct BatchDesc {
    TiledKernel<S, LES, NXC> K;
    S *buf[2];          // population buffers; the old one is buf[step & 1]
    int ntiles;         // work items of this solve per step
};

template <class S, bool LES, int NXC>
__global__ void __launch_bounds__(NTHREADS, 2) step_tiled_kernel(TiledKernel<S, LES, NXC> K) { K.run(); }

template <class S, bool LES, int NXC>
__global__ void __launch_bounds__(NTHREADS, 2)
step_tiled_batch_kernel(const BatchDesc<S, LES, NXC> *__restrict__ descs, const int2 *__restrict__ items, int nitems,
                        int macros_on) {
    using KT = TiledKernel<S, LES, NXC>;
    using LY = Lay<S, NXC>;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(16) unsigned char kbuf[sizeof(KT)];
    __shared__ unsigned long long step_s;
    KT &K = *(KT *)kbuf;
    uint64_t *bars = (uint64_t *)(smem + LY::bar_off);
    const int tid = threadIdx.x;
    if (tid == 0) {
        for (int s = 0; s < LY::NS; s++) mbar_init(&bars[s], 1);
        *(volatile int *)(smem + LY::flag_off) = 0;
        fence_mbar_init();
    }
    unsigned parity = 0;
    bool faulted = false;
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        const int2 w = items[it];   // (solve, tile)
        __syncthreads();            // previous item done with K and every stage
        {
            const unsigned *src = (const unsigned *)&descs[w.x].K;
            unsigned *dst = (unsigned *)kbuf;
            for (int i = tid; i < (int)(sizeof(KT)/4); i += NTHREADS) dst[i] = src[i];
        }
        if (tid == 0) step_s = *(volatile unsigned long long *)&descs[w.x].K.ctrl->step;
        __syncthreads();
        if (tid == 0) {
            const unsigned long long st = step_s;
            K.fo = descs[w.x].buf[st & 1ULL];
            K.fn = descs[w.x].buf[(st + 1) & 1ULL];
            K.tc.n = st + 1;
            K.mass_on = K.k.mass_interval > 0 && ((st + 1) % (unsigned long long)K.k.mass_interval) == 0ULL;
            K.macros_on = macros_on;
        }
        __syncthreads();
        const auto L = K.lane();
        const auto sc = K.scalars();
        Ring R;
        float ub = 0.f, mass = 0.f;
        K.column(w.y, smem, R, parity, faulted, L, sc, ub, mass);
        end_of_step<NTHREADS>(K.ctrl, K.k, K.tc.n, (double)ub, (double)mass, true, K.mass_on != 0,
                              (unsigned)descs[w.x].ntiles);
    }
    __syncthreads();
    if (nitems > 0) K.drain(smem, parity, tid);
}

template <class S, bool LES, int NXC>
cudaError_t launch_t(const StepLaunch &L) {
    TiledKernel<S, LES, NXC> K;
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
    static bool attr_done = false;   // one attribute call per instantiation
    constexpr size_t smem = Lay<S, NXC>::smem_bytes;
    if (!attr_done) {
        cudaError_t e = cudaFuncSetAttribute(step_tiled_kernel<S, LES, NXC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr_done = true;
    }
    step_tiled_kernel<S, LES, NXC><<<K.tc.grid, NTHREADS, smem, L.stream>>>(K);
    return cudaGetLastError();
}

template <class S, bool LES>
cudaError_t launch_nx(const StepLaunch &L) {
    switch (L.k.NX) {
    case 32: return launch_t<S, LES, 32>(L);
    case 64: return launch_t<S, LES, 64>(L);
    default: return launch_t<S, LES, 128>(L);
    }
}

template <class S>
cudaError_t launch_s(const StepLaunch &L) {
    return L.les ? launch_nx<S, true>(L) : launch_nx<S, false>(L);
}

template <class S>
size_t smem_for(int nx) {
    return nx == 32 ? Lay<S, 32>::smem_bytes : (nx == 64 ? Lay<S, 64>::smem_bytes : Lay<S, 128>::smem_bytes);
}

size_t elem_bytes(int precision) { return precision == ISLBM_FP32 ? 4 : 2; }

}  // namespace

bool tiled_supported(const StepConst &k, int precision) {
    if (precision == ISLBM_FP64) return false;
    // spanwise widths with a compiled layout (a tile is 256 nodes)
    if (k.NX != 32 && k.NX != 64 && k.NX != 128) return false;
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
    tc.ybuf_off = 2*tc.stage_bytes;
    tc.xbuf_off = tc.ybuf_off + (size_t)4*tc.TY*k.NX*sizeof(float);
    tc.bar_off = tc.xbuf_off + (size_t)10*tc.TY*k.NX*sizeof(float);
    tc.smem_bytes = precision == ISLBM_FP32 ? smem_for<float>(k.NX) : smem_for<__half>(k.NX);
    for (int a = 0; a < 7; a++) {
        tc.wx0[a] = (float)wx0[a]; tc.wx2[a] = (float)wx2[a];
        tc.wy0[a] = (float)wy0[a]; tc.wy2[a] = (float)wy2[a];
    }
    const int tiles = k.NY/tc.TY;
    tc.units = (long long)tiles*k.NZ;
    tc.grid = tiles < 2*num_sms ? tiles : 2*num_sms;   // two CTAs per SM
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

namespace {

template <class T> struct TypeTag { using type = T; };

template <class S, bool LES, int NXC>
struct BatchOps {
    using D = BatchDesc<S, LES, NXC>;
    static size_t bytes() { return sizeof(D); }
    static void fill(const Tables<float> &T, const StepConst &k, const TiledConst &tc, Ctrl *ctrl, void *const macros[4],
                     void *buf0, void *buf1, int ntiles, void *out) {
        D d;
        std::memset((void *)&d, 0, sizeof(d));
        d.K.T = T; d.K.k = k; d.K.tc = tc; d.K.ctrl = ctrl;
        d.K.rho_out = (float *)macros[0]; d.K.u_out = (float *)macros[1];
        d.K.v_out = (float *)macros[2]; d.K.w_out = (float *)macros[3];
        d.buf[0] = (S *)buf0; d.buf[1] = (S *)buf1;
        d.ntiles = ntiles;
        std::memcpy(out, (const void *)&d, sizeof(d));
    }
    static cudaError_t prepare() {
        static bool attr_done = false;
        if (!attr_done) {
            cudaError_t e = cudaFuncSetAttribute(step_tiled_batch_kernel<S, LES, NXC>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)Lay<S, NXC>::smem_bytes);
            if (e != cudaSuccess) return e;
            attr_done = true;
        }
        return cudaSuccess;
    }
    static cudaError_t launch(const void *descs, const int2 *items, int nitems, int grid, int macros_on, cudaStream_t st) {
        cudaError_t e = prepare();
        if (e != cudaSuccess) return e;
        step_tiled_batch_kernel<S, LES, NXC><<<grid, NTHREADS, Lay<S, NXC>::smem_bytes, st>>>((const D *)descs, items,
                                                                                             nitems, macros_on);
        return cudaGetLastError();
    }
};

template <class F>
auto dispatch(int precision, int NX, bool les, F &&f) {
    auto by_nx = [&](auto s_tag, auto les_tag) {
        using S = typename decltype(s_tag)::type;
        constexpr bool L = decltype(les_tag)::value;
        switch (NX) {
        case 32: return f(BatchOps<S, L, 32>{});
        case 64: return f(BatchOps<S, L, 64>{});
        default: return f(BatchOps<S, L, 128>{});
        }
    };
    auto by_les = [&](auto s_tag) {
        return les ? by_nx(s_tag, std::true_type{}) : by_nx(s_tag, std::false_type{});
    };
    switch (precision) {
    case ISLBM_FP32: return by_les(TypeTag<float>{});
    case ISLBM_FP16_DEV: return by_les(TypeTag<__half>{});
    default: return by_les(TypeTag<__nv_bfloat16>{});
    }
}

}  // namespace

size_t batch_desc_bytes(int precision, int NX, bool les) {
    return dispatch(precision, NX, les, [](auto ops) { return decltype(ops)::bytes(); });
}

void fill_batch_desc(int precision, int NX, bool les, const Tables<float> &T, const StepConst &k, const TiledConst &tc,
                     Ctrl *ctrl, void *const macros[4], void *buf0, void *buf1, int ntiles, void *out) {
    dispatch(precision, NX, les, [&](auto ops) {
        decltype(ops)::fill(T, k, tc, ctrl, macros, buf0, buf1, ntiles, out);
        return 0;
    });
}

cudaError_t prepare_step_tiled_batch(int precision, int NX, bool les) {
    return dispatch(precision, NX, les, [&](auto ops) { return decltype(ops)::prepare(); });
}

cudaError_t launch_step_tiled_batch(int precision, int NX, bool les, const void *descs, const int2 *items, int nitems,
                                    int grid, int macros_on, cudaStream_t stream) {
    return dispatch(precision, NX, les,
                    [&](auto ops) { return decltype(ops)::launch(descs, items, nitems, grid, macros_on, stream); });
}

}  // namespace islbm
