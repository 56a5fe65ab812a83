// Paired tiled step kernel: the tiled z-marching step with two threads per node.
//
// Same step as stream_collide (C/evolution.h:358-684) and the same arithmetic, in the same
// order, as step_tiled.cu; the difference is how the work of a node is split. A CTA of 256
// threads owns a tile of 128 nodes (TY = 128/NX full-width rows) and marches up its column:
//   * role A (warps 0-3) carries directions 1, 3-10 and role B (warps 4-7) directions 2,
//     11-18 through the streamwise / spanwise filters and the xi combination, so each thread
//     keeps a 7-plane register ring of 8 directions instead of 16 and twice as many warps
//     fit on an SM (the ring is the register bound of the one-thread-per-node form);
//   * directions 1 and 2 (spanwise only, no xi) are filtered at the target plane itself,
//     whose f1/f2 rows ride in the stage with the target's xi weights and f0 row;
//   * the streamed populations of a target are exchanged through shared memory and the
//     collision of two consecutive targets is shared: at every odd target plane, role A
//     collides the previous target and role B the current one, one node per thread.
// Copies are cp.async.bulk into a 2-stage ring tracked by mbarriers with bounded waits.
#include <cstring>
#include <type_traits>

#include "step_common.cuh"
#include "step_launch.hpp"
#include "step_tiled.hpp"
#include "tile_helpers.cuh"

namespace islbm {

namespace {

constexpr int PT = 256;         // threads per CTA
constexpr int PN = 128;         // nodes per tile
constexpr int PSTAGES = 2;

// Shared-memory layout for spanwise width NXC: stage s holds populations 3..18 of one plane
// (rows(q) rows each: TY, or TY + 6 with the streamwise halo), then the target's xi weights
// (TY x 64 floats) and its f0, f1, f2 rows; then ybuf [4][PN] (dirs 7..10 after the
// streamwise filter), xbuf [8][PN] (dirs 7..14 after the spanwise filter), fbuf [2][19][PN]
// (streamed populations of two targets), the stage mbarriers.
template <class S, int NXC>
struct LayP {
    static constexpr int NX = NXC;
    static constexpr int TY = PN/NXC;
    static constexpr int LOG2NX = NXC == 32 ? 5 : NXC == 64 ? 6 : 7;
    static constexpr int EB = (int)sizeof(S);
    static constexpr bool wide(int q) { return q == 3 || q == 4 || (q >= 7 && q <= 10) || q >= 15; }
    static constexpr int rows(int q) { return q <= 2 ? 0 : (wide(q) ? TY + 6 : TY); }
    static constexpr int up16(int v) { return (v + 15)/16*16; }
    static constexpr int off_bytes(int q) {
        int off = 0;
        for (int r = 3; r < q; ++r) off = up16(off + rows(r)*NX*EB);
        return off;
    }
    static constexpr int off(int q) { return off_bytes(q)/EB; }
    static constexpr unsigned pops_bytes() {
        unsigned b = 0;
        for (int q = 3; q < 19; ++q) b += (unsigned)(rows(q)*NX*EB);
        return b;
    }
    static constexpr int w_off = off_bytes(19);
    static constexpr int f0_off = up16(w_off + TY*64*4);
    static constexpr int f1_off = up16(f0_off + TY*NX*EB);
    static constexpr int f2_off = up16(f1_off + TY*NX*EB);
    static constexpr int stage_bytes = (up16(f2_off + TY*NX*EB) + 127)/128*128;
    static constexpr unsigned tgt_bytes = (unsigned)(TY*64*4 + 3*TY*NX*EB);
    static constexpr int ybuf_off = PSTAGES*stage_bytes;
    static constexpr int xbuf_off = ybuf_off + 4*PN*4;
    static constexpr int fbuf_off = xbuf_off + 8*PN*4;
    static constexpr int bar_off = fbuf_off + 2*19*PN*4;
    static constexpr int smem_bytes = bar_off + PSTAGES*8;
};

// Filtered values of one plane for one role: A (r34, r56, r78, r910), B (r1112, r1314, r1516,
// r1718).
struct HSlot {
    float2 a, b, c, d;
};
struct HRing {
    HSlot s[7];
};

// xi combination of the window whose newest plane sits in slot NEW; out = the role's 8
// directions in pair order. Weights per stencil point c: (xi3, xi4, xi5, xi6 | xi15, xi16, xi17,
// xi18), the same interleave and FMA order as the one-thread-per-node kernel.
template <int NEW, int ROLE>
__device__ __forceinline__ void hcombine(const HRing &R, const float *wv_, float *out) {
    const float4 *wv = (const float4 *)wv_;
    constexpr int O = (NEW + 1) % 7;
    P2 x = p2(0.f, 0.f), y = x, z = x, t = x;
#pragma unroll
    for (int c = 0; c < 7; c++) {
        const HSlot &q = R.s[(O + c) % 7];
        const float4 w = wv[2*c];
        if constexpr (ROLE == 0) {
            fma2(x, p2(w.x, w.y), p2(q.a));   // 3, 4
            fma2(y, p2(w.z, w.w), p2(q.b));   // 5, 6
            fma2(z, p2(w.x, w.x), p2(q.c));   // 7, 8
            fma2(t, p2(w.y, w.y), p2(q.d));   // 9, 10
        } else {
            const float4 u = wv[2*c + 1];
            fma2(x, p2(w.z, w.z), p2(q.a));   // 11, 12
            fma2(y, p2(w.w, w.w), p2(q.b));   // 13, 14
            fma2(z, p2(u.x, u.y), p2(q.c));   // 15, 16
            fma2(t, p2(u.z, u.w), p2(q.d));   // 17, 18
        }
    }
    float2 r;
    r = unp(x); out[0] = r.x; out[1] = r.y;
    r = unp(y); out[2] = r.x; out[3] = r.y;
    r = unp(z); out[4] = r.x; out[5] = r.y;
    r = unp(t); out[6] = r.x; out[7] = r.y;
}

template <int ROLE>
__device__ __forceinline__ void hcombine_phase(int ph, const HRing &R, const float *wv, float *out) {
    switch (ph) {
    case 0: hcombine<0, ROLE>(R, wv, out); break;
    case 1: hcombine<1, ROLE>(R, wv, out); break;
    case 2: hcombine<2, ROLE>(R, wv, out); break;
    case 3: hcombine<3, ROLE>(R, wv, out); break;
    case 4: hcombine<4, ROLE>(R, wv, out); break;
    case 5: hcombine<5, ROLE>(R, wv, out); break;
    default: hcombine<6, ROLE>(R, wv, out); break;
    }
}

__device__ __forceinline__ void hring_store(HRing &R, int ph, const HSlot &v) {
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
struct PairKernel {
    using LY = LayP<S, NXC>;
    struct Scal { float f6, f12, rho_mod, tau, lesC; };
    const S *__restrict__ fo;
    S *__restrict__ fn;
    Tables<float> T;
    StepConst k;
    TiledConst tc;
    Ctrl *ctrl;
    float *rho_out, *u_out, *v_out, *w_out;
    int macros_on, mass_on;

    struct Lane {
        int tid, role, n, xl, yl;    // role 0 = A, 1 = B; node n of the tile
        int t0r, t0x;                // spanwise task 0 (dirs 7..10 from ybuf): row, first node
        int t1r, t1x;                // spanwise task 1 (dirs 11..14 from the stage)
        int t0d, t1d;                // xbuf slots of the two tasks (0..3, 4..7)
        int t1off;                   // stage offset (elements) of task 1's population
    };

    __device__ __forceinline__ Lane lane() const {
        constexpr int NX = LY::NX;
        Lane L;
        L.tid = threadIdx.x;
        L.role = L.tid >> 7;
        L.n = L.tid & (PN - 1);
        L.xl = L.n & (NX - 1);
        L.yl = L.n >> LY::LOG2NX;
        // 512 two-node tasks per plane: (xbuf slot d, pair) with 64 pairs per slot
        const int pair = L.tid & 63;
        L.t0d = L.tid >> 6;
        L.t1d = 4 + (L.tid >> 6);
        L.t0r = L.t1r = pair >> (LY::LOG2NX - 1);
        L.t0x = L.t1x = 2*(pair & (NX/2 - 1));
        switch (L.t1d) {   // warp-uniform
        case 4: L.t1off = LY::off(11); break;
        case 5: L.t1off = LY::off(12); break;
        case 6: L.t1off = LY::off(13); break;
        default: L.t1off = LY::off(14); break;
        }
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

    // Walls, BFL rows, collision and store of one node (F[1..18] filtered values, deviations
    // for the deviation formats; F[0] full).
    __device__ __forceinline__ void finish(float *F, int x, int y, int z, const Scal &sc, float &ub, float &mass) const {
        constexpr int NX = LY::NX;
        const int NY = k.NY;
        const size_t N = (size_t)NX*NY*k.NZ;
        const size_t node = ((size_t)z*NY + y)*NX + x;
        if constexpr (Storage<S>::dev) {
#pragma unroll
            for (int q = 1; q < 19; q++) F[q] += lattice_w<float>(q);
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
        collide_node<float, LES>(*(float(*)[19])F, sc.rho_mod, sc.f6, sc.f12, sc.tau, sc.lesC, rho_s, u1, v1, w1);
#pragma unroll
        for (int q = 0; q < 19; q++) store_f<S>(fn + (size_t)q*N, node, q, F[q]);
        if (macros_on) { rho_out[node] = rho_s; u_out[node] = u1; v_out[node] = v1; w_out[node] = w1; }
        if (y == k.yplane) ub += v1*T.dxf[x]*T.dzf[z];
        mass += rho_s;
        if (!(rho_s == rho_s)) ctrl->nonfinite = 1u;
    }

    // Warp 0: expected bytes, then lane q copies population q (3..18, two pieces when the halo
    // wraps) and lanes 19..22 the target data (xi weights, f0, f1, f2 rows of plane p - 3).
    __device__ void issue_plane(unsigned char *stage, uint64_t *bar, int p, int y0, int lane) const {
        constexpr int NX = LY::NX, TY = LY::TY;
        const int NY = k.NY, NZ = k.NZ;
        const size_t N = (size_t)NX*NY*NZ;
        const unsigned row_bytes = (unsigned)(NX*sizeof(S));
        const bool tgt = p >= 7 && p <= NZ - 1;
        if (lane == 0) mbar_expect_tx(bar, LY::pops_bytes() + (tgt ? LY::tgt_bytes : 0u));
        __syncwarp();
        S *pops = (S *)stage;
        const int q = lane;
        if (q >= 3 && q < 19) {
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
        if (tgt) {
            const int z = p - 3;
            if (lane == 19)
                bulk_g2s(stage + LY::w_off, T.wxi + ((size_t)z*NY + y0)*64, (unsigned)(TY*64*sizeof(float)), bar);
            if (lane >= 20 && lane <= 22) {
                const int qq = lane - 20;   // f0, f1, f2
                const int o = qq == 0 ? LY::f0_off : (qq == 1 ? LY::f1_off : LY::f2_off);
                bulk_g2s(stage + o, fo + (size_t)qq*N + ((size_t)z*NY + y0)*NX, TY*row_bytes, bar);
            }
        }
    }

    __device__ __forceinline__ void issue(unsigned char *smem, int s, int p, int y0, const Lane &L, unsigned &parity,
                                          bool faulted) const {
        if (__any_sync(0xffffffffu, faulted)) return;
        fence_proxy_async();
        issue_plane(smem + (size_t)s*LY::stage_bytes, (uint64_t *)(smem + LY::bar_off) + s, p, y0, L.tid);
        parity = (parity & ~(1u << (PPAR + s))) | (((parity >> s) & 1u) << (PPAR + s)) | (1u << (PEND + s));
    }

    __device__ __forceinline__ void drain(unsigned char *smem, unsigned parity, int tid) const {
        if (tid >= 32) return;
        uint64_t *bars = (uint64_t *)(smem + LY::bar_off);
        for (int s = 0; s < PSTAGES; s++) {
            if (!((parity >> (PEND + s)) & 1u)) continue;
            const unsigned ph = (parity >> (PPAR + s)) & 1u;
            for (int it = 0; it < (1 << 22); ++it) {
                if (mbar_try_wait(&bars[s], ph)) break;
                if (it > 32) __nanosleep(256);
            }
        }
    }

    // One source plane: wait for its copies, filter, return this role's slot values.
    __device__ __forceinline__ HSlot plane(int i, int p, int p1, int y0, unsigned char *smem, unsigned &parity,
                                           bool &faulted, const Lane &L) const {
        constexpr int NX = LY::NX;
        const int s = i % PSTAGES;
        uint64_t *bars = (uint64_t *)(smem + LY::bar_off);
        float *ybuf = (float *)(smem + LY::ybuf_off);   // [4][PN]  dirs 7, 8, 9, 10
        float *xbuf = (float *)(smem + LY::xbuf_off);   // [8][PN]  dirs 7..14
        unsigned char *stage = smem + (size_t)s*LY::stage_bytes;
        const S *raw = (const S *)stage;
        if (mbar_wait(&bars[s], (parity >> s) & 1u, ctrl, faulted)) parity &= ~(1u << (PEND + s));
        parity ^= 1u << s;
        HSlot v;
        {   // streamwise filter over rows yl .. yl+6 of the halo copy
            const S *base = raw + L.yl*NX + L.xl;
            auto row = [&](int q, int b) -> const S * { return base + LY::off(q) + b*NX; };
            if (L.role == 0) {
                float a3 = 0, a4 = 0, a7 = 0, a8 = 0, a9 = 0;
#pragma unroll
                for (int b = 0; b < 7; b++) {
                    const float y0w = tc.wy0[b], y2w = tc.wy2[b];
                    a3 += y0w*ldv<S>(row(3, b)); a4 += y2w*ldv<S>(row(4, b));
                    a7 += y0w*ldv<S>(row(7, b)); a8 += y0w*ldv<S>(row(8, b));
                    a9 += y2w*ldv<S>(row(9, b));
                }
                v.a = make_float2(a3, a4);
                v.b = make_float2(ldv<S>(row(5, 0)), ldv<S>(row(6, 0)));
                ybuf[0*PN + L.n] = a7; ybuf[1*PN + L.n] = a8; ybuf[2*PN + L.n] = a9;
            } else {
                float a10 = 0, a15 = 0, a16 = 0, a17 = 0, a18 = 0;
#pragma unroll
                for (int b = 0; b < 7; b++) {
                    const float y0w = tc.wy0[b], y2w = tc.wy2[b];
                    a10 += y2w*ldv<S>(row(10, b));
                    a15 += y0w*ldv<S>(row(15, b)); a16 += y2w*ldv<S>(row(16, b));
                    a17 += y0w*ldv<S>(row(17, b)); a18 += y2w*ldv<S>(row(18, b));
                }
                v.c = make_float2(a15, a16);
                v.d = make_float2(a17, a18);
                ybuf[3*PN + L.n] = a10;
            }
        }
        __syncthreads();
        // every thread has finished plane i-1: its stage can take plane i + PSTAGES - 1
        if (L.tid < 32 && p + PSTAGES - 1 <= p1) issue(smem, (i + PSTAGES - 1) % PSTAGES, p + PSTAGES - 1, y0, L, parity, faulted);
        {   // spanwise filter, two tasks of two nodes: dirs 7..10 from ybuf, dirs 11..14 raw
            const int m = NX - 1;
            auto xf = [&](int d, const float2 (&vv)[5], int r, int x0) {
                float o0 = 0, o1 = 0;
                const float e[10] = {vv[0].x, vv[0].y, vv[1].x, vv[1].y, vv[2].x, vv[2].y, vv[3].x, vv[3].y, vv[4].x, vv[4].y};
#pragma unroll
                for (int a = 0; a < 7; a++) {
                    const float w = (d & 1) ? tc.wx2[a] : tc.wx0[a];
                    o0 += w*e[a + 1]; o1 += w*e[a + 2];
                }
                *(float2 *)(xbuf + (size_t)d*PN + r*NX + x0) = make_float2(o0, o1);
            };
            {
                const int x0 = L.t0x;
                const float *in = ybuf + (size_t)L.t0d*PN + L.t0r*NX;
                const float2 vv[5] = {*(const float2 *)(in + ((x0 - 4) & m)), *(const float2 *)(in + ((x0 - 2) & m)),
                                      *(const float2 *)(in + x0), *(const float2 *)(in + ((x0 + 2) & m)),
                                      *(const float2 *)(in + ((x0 + 4) & m))};
                xf(L.t0d, vv, L.t0r, x0);
            }
            {
                const int x0 = L.t1x;
                const S *in = raw + L.t1off + L.t1r*NX;
                const float2 vv[5] = {ldv2<S>(in + ((x0 - 4) & m)), ldv2<S>(in + ((x0 - 2) & m)), ldv2<S>(in + x0),
                                      ldv2<S>(in + ((x0 + 2) & m)), ldv2<S>(in + ((x0 + 4) & m))};
                xf(L.t1d, vv, L.t1r, x0);
            }
        }
        __syncthreads();
        if (L.role == 0) {
            v.c = make_float2(xbuf[0*PN + L.n], xbuf[1*PN + L.n]);
            v.d = make_float2(xbuf[2*PN + L.n], xbuf[3*PN + L.n]);
        } else {
            v.a = make_float2(xbuf[4*PN + L.n], xbuf[5*PN + L.n]);
            v.b = make_float2(xbuf[6*PN + L.n], xbuf[7*PN + L.n]);
        }
        return v;
    }

    // this role's streamed values of a target into fbuf slot (z & 1)
    __device__ __forceinline__ void put(unsigned char *smem, int z, const Lane &L, const float *o8, float f12, float f0) const {
        float *fb = (float *)(smem + LY::fbuf_off) + (size_t)(z & 1)*19*PN + L.n;
        if (L.role == 0) {
            fb[0*PN] = f0; fb[1*PN] = f12;
#pragma unroll
            for (int j = 0; j < 8; j++) fb[(3 + j)*PN] = o8[j];
        } else {
            fb[2*PN] = f12;
#pragma unroll
            for (int j = 0; j < 8; j++) fb[(11 + j)*PN] = o8[j];
        }
    }

    // collide the target in fbuf slot `slot` (plane z) at this thread's node
    __device__ __forceinline__ void collide_slot(unsigned char *smem, int slot, int z, int y0, const Lane &L,
                                                 const Scal &sc, float &ub, float &mass) const {
        const float *fb = (const float *)(smem + LY::fbuf_off) + (size_t)slot*19*PN + L.n;
        float F[19];
#pragma unroll
        for (int q = 0; q < 19; q++) F[q] = fb[q*PN];
        finish(F, L.xl, y0 + L.yl, z, sc, ub, mass);
    }

    // after target z has been put: once two targets are pending, every thread collides one
    __device__ __forceinline__ void after_put(unsigned char *smem, int z, int y0, const Lane &L, const Scal &sc, float &ub,
                                              float &mass) const {
        __syncthreads();
        if (z & 1) collide_slot(smem, L.role, z - 1 + L.role, y0, L, sc, ub, mass);
    }

    // F1 (role A) or F2 (role B) of a wall-cap target by direct spanwise gathers
    __device__ __forceinline__ float cap_f12(int x, int y, int z, int role) const {
        constexpr int NX = LY::NX;
        const int NY = k.NY;
        const size_t N = (size_t)NX*NY*k.NZ;
        const S *r = fo + (size_t)(1 + role)*N + ((size_t)z*NY + y)*NX;
        float a = 0;
#pragma unroll
        for (int t = 0; t < 7; t++) a += (role ? tc.wx2[t] : tc.wx0[t])*ldv<S>(r + ((x - 3 + t) & (NX - 1)));
        return a;
    }

    __device__ __forceinline__ void cap_target(unsigned char *smem, const HRing &R, int ph, int z, int y0, const Lane &L,
                                               const Scal &sc, float &ub, float &mass) const {
        const int y = y0 + L.yl;
        float o8[8];
        const float *wv = T.wxi + ((size_t)z*k.NY + y)*64;
        if (L.role == 0) hcombine_phase<0>(ph, R, wv, o8); else hcombine_phase<1>(ph, R, wv, o8);
        const float f12 = cap_f12(L.xl, y, z, L.role);
        const float f0 = L.role == 0 ? load_f<S>(fo, ((size_t)z*k.NY + y)*LY::NX + L.xl, 0) : 0.f;
        __syncthreads();   // the previous collision has read fbuf
        put(smem, z, L, o8, f12, f0);
        after_put(smem, z, y0, L, sc, ub, mass);
    }

    __device__ __forceinline__ void column(int tile, unsigned char *smem, HRing &R, unsigned &parity, bool &faulted,
                                           const Lane &L, const Scal &sc, float &ub, float &mass) const {
        constexpr int NX = LY::NX, TY = LY::TY;
        const int NZ = k.NZ;
        const int y0 = tile*TY;
        const int p1 = NZ - 1;
        __syncthreads();   // every thread is done with every stage and fbuf of the previous column
        if (L.tid < 32)
            for (int s = 0; s < PSTAGES - 1 && s <= p1; s++) issue(smem, s, s, y0, L, parity, faulted);
        // planes 0..6 fill the ring (plane p in slot p mod 7); then the lower cap
#pragma unroll 1
        for (int p = 0; p < 7; p++) {
            const HSlot v = plane(p, p, p1, y0, smem, parity, faulted, L);
            hring_store(R, p, v);
        }
        for (int zt = 0; zt < 4; zt++) cap_target(smem, R, 6, zt, y0, L, sc, ub, mass);
        // steady state: each plane completes the window of one interior target
        int ph = 0;
#pragma unroll 1
        for (int p = 7; p <= NZ - 1; p++) {
            const HSlot v = plane(p, p, p1, y0, smem, parity, faulted, L);
            hring_store(R, ph, v);
            const unsigned char *stage = smem + (size_t)(p % PSTAGES)*LY::stage_bytes;
            const float *wv = (const float *)(stage + LY::w_off) + L.yl*64;
            float o8[8];
            if (L.role == 0) hcombine_phase<0>(ph, R, wv, o8); else hcombine_phase<1>(ph, R, wv, o8);
            // F1 / F2 at the target plane: spanwise filter straight from the staged row
            const S *r12 = (const S *)(stage + (L.role ? LY::f2_off : LY::f1_off)) + L.yl*NX;
            float f12 = 0;
#pragma unroll
            for (int t = 0; t < 7; t++) f12 += (L.role ? tc.wx2[t] : tc.wx0[t])*ldv<S>(r12 + ((L.xl - 3 + t) & (NX - 1)));
            const float f0 = ld1<S>((const S *)(stage + LY::f0_off) + L.yl*NX + L.xl, 1.f/3);
            put(smem, p - 3, L, o8, f12, f0);
            after_put(smem, p - 3, y0, L, sc, ub, mass);
            ph = ph == 6 ? 0 : ph + 1;
        }
        const int phl = (NZ - 1) % 7;
        for (int zt = NZ - 3; zt < NZ; zt++) cap_target(smem, R, phl, zt, y0, L, sc, ub, mass);
        if (NZ & 1) {   // the last target (even plane) is still pending: role A collides it
            if (L.role == 0) collide_slot(smem, 0, NZ - 1, y0, L, sc, ub, mass);
        }
    }

    __device__ void run() const {
        extern __shared__ __align__(128) unsigned char smem[];
        uint64_t *bars = (uint64_t *)(smem + LY::bar_off);
        const Lane L = lane();
        if (L.tid == 0) {
            for (int s = 0; s < PSTAGES; s++) mbar_init(&bars[s], 1);
            fence_mbar_init();
        }
        __syncthreads();
        unsigned parity = 0;
        bool faulted = false;
        double ub_total = 0.0, mass_total = 0.0;
        const Scal sc = scalars();
        HRing R;
        const int ntiles = k.NY/LY::TY;
        for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
            float ub = 0.f, mass = 0.f;
            column(tile, smem, R, parity, faulted, L, sc, ub, mass);
            ub_total += (double)ub;
            mass_total += (double)mass;
        }
        drain(smem, parity, L.tid);
        end_of_step<PT>(ctrl, k, tc.n, ub_total, mass_total, true, mass_on != 0, gridDim.x*gridDim.y*gridDim.z);
    }
};

template <class S, bool LES, int NXC>
__global__ void __launch_bounds__(PT, 2) step_pair_kernel(PairKernel<S, LES, NXC> K) { K.run(); }

template <class S, bool LES, int NXC>
cudaError_t launch_p(const StepLaunch &L) {
    PairKernel<S, LES, NXC> K;
    K.fo = (const S *)L.fo;
    K.fn = (S *)L.fn;
    K.T = *(const Tables<float> *)L.tables;
    K.k = L.k;
    K.tc = *(const TiledConst *)L.tiled;
    K.tc.n = L.n;
    K.ctrl = L.ctrl;
    K.rho_out = (float *)L.macros[0]; K.u_out = (float *)L.macros[1];
    K.v_out = (float *)L.macros[2]; K.w_out = (float *)L.macros[3];
    K.macros_on = L.macros_on ? 1 : 0;
    K.mass_on = L.mass ? 1 : 0;
    constexpr int smem = LayP<S, NXC>::smem_bytes;
    static bool attr_done = false;
    if (!attr_done) {
        cudaError_t e = cudaFuncSetAttribute(step_pair_kernel<S, LES, NXC>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        attr_done = true;
    }
    const int ntiles = L.k.NY/LayP<S, NXC>::TY;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int grid = ntiles < 2*sms ? ntiles : 2*sms;
    step_pair_kernel<S, LES, NXC><<<grid, PT, smem, L.stream>>>(K);
    return cudaGetLastError();
}

template <class S, bool LES>
cudaError_t launch_pn(const StepLaunch &L) {
    switch (L.k.NX) {
    case 32: return launch_p<S, LES, 32>(L);
    case 64: return launch_p<S, LES, 64>(L);
    default: return launch_p<S, LES, 128>(L);
    }
}

template <class S>
cudaError_t launch_ps(const StepLaunch &L) {
    return L.les ? launch_pn<S, true>(L) : launch_pn<S, false>(L);
}

}  // namespace

bool pair_supported(const StepConst &k, int precision) {
    if (precision == ISLBM_FP64) return false;
    if (k.NX != 32 && k.NX != 64 && k.NX != 128) return false;
    const int TY = PN/k.NX;
    return k.NY % TY == 0 && k.NY >= TY + 6 && k.NZ >= 8;
}

cudaError_t launch_step_pair(const StepLaunch &L) {
    switch (L.precision) {
    case ISLBM_FP32: return launch_ps<float>(L);
    case ISLBM_FP16_DEV: return launch_ps<__half>(L);
    case ISLBM_BF16_DEV: return launch_ps<__nv_bfloat16>(L);
    default: return cudaErrorNotSupported;
    }
}

}  // namespace islbm
