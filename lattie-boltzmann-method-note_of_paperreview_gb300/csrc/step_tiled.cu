// Tiled step kernel: z-marching x-y tiles staged in shared memory by bulk async copies.
//
// Same step as stream_collide (C/evolution.h:358-684) for FP32 arithmetic with FP32, FP16 or
// BF16 population storage, organised for HBM:
//   * a CTA owns a tile of TY = 128/NX full-width rows (all NX spanwise nodes), one node per
//     thread, and marches upward through a segment of the wall-normal planes of that column;
//     every plane of the 18 moving populations is copied global -> shared with cp.async.bulk
//     (one copy per population and plane, 3-row streamwise halo for the ten populations with
//     e_y != 0, periodic wrap by splitting the copy), tracked by an mbarrier per stage; the
//     target plane's xi weights and f0 row ride in the same stage;
//   * the interpolation is applied as separable filters, exact in real arithmetic because the
//     x and y weights are the same for every node (uniform spacing, C/initialization.h:51-108)
//     and the xi weights depend only on the target (y, z): a streamwise filter over the halo
//     rows, a spanwise filter of each node over its row (streamwise-filtered values exchanged
//     through shared memory), then the xi combination over a 7-plane ring of filtered values
//     kept in tensor memory (TMEM, one lane per thread), all in packed FP32x2 FMAs, so each
//     loaded value feeds 7 target planes without being re-read;
//   * the collision tail, wall bounce-back, BFL rows and controller partial sums are fused;
//   * CTAs are persistent (up to 4 per SM, 128 threads each); work items are (segment, tile)
//     pairs taken segment-major, so the CTAs running at the same time hold neighbouring tiles
//     at similar heights and share the streamwise halo rows through L2.
// Every value of the old populations is read from HBM about once per step (halo rows come
// from L2); every new value is written once.
#include <algorithm>
#include <cstring>
#include <type_traits>

#include "step_common.cuh"
#include "step_launch.hpp"
#include "step_tiled.hpp"
#include "tile_helpers.cuh"

namespace islbm {

namespace {

// Threads per CTA for a spanwise width NXC: one node per thread, at least 128 (tiles of
// 128/NXC full rows), a single row for the widths above 128.
template <int NXC> constexpr int threads_for() { return NXC < 128 ? 128 : NXC; }
// TMEM columns of a CTA's xi ring: 128 per 128 threads (each thread's lane holds 126 values),
// rounded up to a power of two as the allocator requires
template <int NT> constexpr int ring_cols_for() { return NT <= 128 ? 128 : (NT <= 256 ? 256 : 512); }
// Copy stages per tile: the next plane's copies are in flight while one plane is filtered.
template <class S> constexpr int stages_for() { return 2; }

// Shared-memory layout of one tile for a spanwise width NXC (a power of two): all offsets are
// compile-time constants so every shared-memory address is a base plus an immediate.
//   front region (one): the populations read before the first barrier of a plane (the ten
//     with e_y != 0 as TY + 6 rows with the streamwise halo, and 5, 6 as TY rows). All
//     threads are done with it at that barrier, which is where the next plane's copies start,
//     so one buffer overlaps the copies as well as two would;
//   stage s (NS of them): populations 1, 2, 11..14 (TY rows each, read by the spanwise filter
//     after that barrier), then the target's xi weights (TY x 64 floats) and f0 row;
//   then ybuf [2][TY][NXC] float4 (streamwise-filtered 7, 8, 9, 10 of each node, two buffers
//   by plane parity), then the stage mbarriers.
template <class S, int NXC>
struct Lay {
    static constexpr int NX = NXC;
    static constexpr int NT = threads_for<NXC>();
    static constexpr int TY = NT/NXC;
    static constexpr int RING = ring_cols_for<NT>();
    static constexpr int CTAS_PER_SM = 512/RING;   // TMEM bound (512 columns per SM)
    static constexpr int EB = (int)sizeof(S);
    static constexpr int NS = stages_for<S>();
    static constexpr bool wide(int q) { return q == 3 || q == 4 || (q >= 7 && q <= 10) || q >= 15; }
    static constexpr bool front(int q) { return wide(q) || q == 5 || q == 6; }
    static constexpr int rows(int q) { return q == 0 ? 0 : (wide(q) ? TY + 6 : TY); }
    static constexpr int up16(int v) { return (v + 15)/16*16; }
    // byte offset of population q within its region (front or stage)
    static constexpr int off_bytes(int q) {
        int off = 0;
        for (int r = 1; r < q; ++r)
            if (front(r) == front(q)) off = up16(off + rows(r)*NX*EB);
        return off;
    }
    static constexpr int off(int q) { return off_bytes(q)/EB; }
    static constexpr int region_end(bool fr) {
        int off = 0;
        for (int r = 1; r < 19; ++r)
            if (front(r) == fr) off = up16(off + rows(r)*NX*EB);
        return off;
    }
    static constexpr unsigned pops_bytes() {
        unsigned b = 0;
        for (int q = 1; q < 19; ++q) b += (unsigned)(rows(q)*NX*EB);
        return b;
    }
    static constexpr int front_bytes = (region_end(true) + 127)/128*128;
    // front buffers: one for FP32 (four CTAs per SM fit); the 2-byte formats fit two, which keeps
    // the next plane's copy from waiting for the slowest warp's streamwise filter
    static constexpr int NF = EB == 2 ? 2 : 1;
    static constexpr int front_off(int s) { return NF == 1 ? 0 : (s % NF)*front_bytes; }
    static constexpr int w_off = region_end(false);   // within a stage
    static constexpr int f0_off = up16(w_off + TY*64*4);
    static constexpr int stage_bytes = (up16(f0_off + TY*NX*EB) + 127)/128*128;
    static constexpr int stage_off(int s) { return NF*front_bytes + s*stage_bytes; }
    static constexpr unsigned tgt_bytes = (unsigned)(TY*64*4 + TY*NX*EB);
    static constexpr int ybuf_off = NF*front_bytes + NS*stage_bytes;
    static constexpr int bar_off = ybuf_off + 2*TY*NX*16;
    static constexpr int flag_off = bar_off + NS*8;   // CTA-wide "a wait timed out" flag, then the TMEM address
    // large enough that no more than CTAS_PER_SM CTAs fit in an SM's 228 KB (1 KB reserved per
    // CTA), so the TMEM allocations of resident CTAs never exceed the SM's 512 columns
    static constexpr int smem_floor = 228*1024/(CTAS_PER_SM + 1) + 1;
    static constexpr int smem_bytes = flag_off + 16 > smem_floor ? flag_off + 16 : smem_floor;
};

// xi ring in tensor memory: each thread keeps the filtered values of the 7 planes of its
// current window in its own TMEM lane; plane p sits in slot p mod 7:
//   columns 16*s .. 16*s+15: pairs (3,4) (5,6) (15,16) (17,18) (7,9) (8,10) (11,13) (12,14),
//   columns 112 + 2*(p mod 8), +1: the spanwise-filtered F1, F2 of plane p (used by target p,
//   which completes at most three planes later).
// The pairs are chosen so that each pair's xi weights are adjacent in the weight row.
__device__ __forceinline__ int ring_col(int slot) { return 16*slot; }   // slot = p mod 7, tracked by the caller
__device__ __forceinline__ int r12_col(int p) { return 112 + 2*(p & 7); }

// xi combination of the window of planes b .. b+6 held in the TMEM ring (`tl` = this warp's
// lane-quarter address, `sb` = b mod 7). The 64 weights of (y, z) are interleaved per stencil point c:
// (xi3, xi4, xi5, xi6, xi15, xi16, xi17, xi18)[c]. Writes F[3..18], and F[1], F[2] from the
// delay-line columns r12c.
__device__ __forceinline__ void xi_combine(uint32_t tl, int sb, int r12c, const float *wv_, float *F) {
    const float4 *wv = (const float4 *)wv_;
    P2 a34 = p2(0.f, 0.f), a56 = a34, a1516 = a34, a1718 = a34, a79 = a34, a810 = a34, a1113 = a34, a1214 = a34;
    auto acc = [&](const uint32_t (&q)[16], int c) {
        const float4 w = wv[2*c], u = wv[2*c + 1];
        auto pr = [&](int i) { return p2(__uint_as_float(q[i]), __uint_as_float(q[i + 1])); };
        fma2(a34, p2(w.x, w.y), pr(0));
        fma2(a56, p2(w.z, w.w), pr(2));
        fma2(a1516, p2(u.x, u.y), pr(4));
        fma2(a1718, p2(u.z, u.w), pr(6));
        fma2(a79, p2(w.x, w.y), pr(8));
        fma2(a810, p2(w.x, w.y), pr(10));
        fma2(a1113, p2(w.z, w.w), pr(12));
        fma2(a1214, p2(w.z, w.w), pr(14));
    };
#pragma unroll
    for (int c = 0; c < 6; c += 2) {
        uint32_t q0[16], q1[16], r[2];
        const int s0 = sb + c, s1 = sb + c + 1;
        tmem_ld16(tl + ring_col(s0 >= 7 ? s0 - 7 : s0), q0);
        tmem_ld16(tl + ring_col(s1 >= 7 ? s1 - 7 : s1), q1);
        if (c == 0) tmem_ld2(tl + r12c, r);   // F1, F2 of the target plane ride with the first pair
        tmem_wait_ld(q0, q1);
        if (c == 0) {
            tmem_tie(r);
            F[1] = __uint_as_float(r[0]); F[2] = __uint_as_float(r[1]);
        }
        acc(q0, c);
        acc(q1, c + 1);
    }
    {   // the newest plane: its ring stores were issued by this thread just before
        uint32_t q0[16];
        tmem_wait_st();
        tmem_ld16(tl + ring_col(sb == 0 ? 6 : sb - 1), q0);
        tmem_wait_ld(q0);
        acc(q0, 6);
    }
    float2 t;
    t = unp(a34); F[3] = t.x; F[4] = t.y;
    t = unp(a56); F[5] = t.x; F[6] = t.y;
    t = unp(a1516); F[15] = t.x; F[16] = t.y;
    t = unp(a1718); F[17] = t.x; F[18] = t.y;
    t = unp(a79); F[7] = t.x; F[9] = t.y;
    t = unp(a810); F[8] = t.x; F[10] = t.y;
    t = unp(a1113); F[11] = t.x; F[13] = t.y;
    t = unp(a1214); F[12] = t.x; F[14] = t.y;
}

// periodic spanwise index for v in [-NX, 2*NX)
template <int NX> __device__ __forceinline__ int wrap_x(int v) {
    if constexpr ((NX & (NX - 1)) == 0) return v & (NX - 1);
    else return v < 0 ? v + NX : (v >= NX ? v - NX : v);
}

template <class S, bool LES, int NXC>
struct TiledKernel {
    using LY = Lay<S, NXC>;
    // per-launch float constants (computed once per thread from the FP64 controller state)
    struct Scal { float f6, f12, rho_mod, tau, lesC; };
    const S *__restrict__ fo;
    S *__restrict__ fn;
    S *fnq[19];                // fn + q*N: per-direction bases, so a store is base + 32-bit node index
    Tables<float> T;
    StepConst k;
    TiledConst tc;
    Ctrl *ctrl;
    float *rho_out, *u_out, *v_out, *w_out;
    int macros_on, mass_on;

    // Walls, BFL rows, collision and store of one node whose streamed populations are in F
    // (F[1..18] as filtered values, deviations for the deviation formats; F[0] full).
    // CAP: a wall-cap target (z <= 3 or z >= NZ-4), the only ones that can be wall rows (bounce-back
    // at z = 0 and NZ-1, BFL rows at z <= 1).
    template <bool CAP>
    __device__ __forceinline__ void finish(float *F, int x, int y, int z, const Scal &sc, float &ub, float &mass) const {
        constexpr int NX = LY::NX;
        const int NY = k.NY;
        const size_t N = (size_t)NX*NY*k.NZ;
        const size_t node = ((size_t)z*NY + y)*NX + x;
        if constexpr (Storage<S>::dev) {
#pragma unroll
            for (int q = 1; q < 19; q++) F[q] += (float)dev_ref(q);
        }
        if (CAP && z == 0) {
            const S *b = fo + node;
            F[5] = load_f<S>(b + 6*N, 0, 6); F[11] = load_f<S>(b + 14*N, 0, 14); F[12] = load_f<S>(b + 13*N, 0, 13);
            F[15] = load_f<S>(b + 18*N, 0, 18); F[16] = load_f<S>(b + 17*N, 0, 17);
        }
        if (CAP && z == k.NZ - 1) {
            const S *b = fo + node;
            F[6] = load_f<S>(b + 5*N, 0, 5); F[13] = load_f<S>(b + 12*N, 0, 12); F[14] = load_f<S>(b + 11*N, 0, 11);
            F[17] = load_f<S>(b + 16*N, 0, 16); F[18] = load_f<S>(b + 15*N, 0, 15);
        }
        if (CAP && z <= 1) {
            const int nb = 2*k.NYD6, r = z*k.NYD6 + (y + 3);
            if (T.bfl_flag[r] | T.bfl_flag[nb + r] | T.bfl_flag[2*nb + r] | T.bfl_flag[3*nb + r]) {
                // the out-of-line BFL rows work on a copy, so that F itself never needs an address
                float G[19];
#pragma unroll
                for (int q = 0; q < 19; q++) G[q] = F[q];
                bfl_node<S>(fo, T, k, x, y, z, G);
#pragma unroll
                for (int q = 0; q < 19; q++) F[q] = G[q];
            }
        }
        float Fl[19];
#pragma unroll
        for (int q = 0; q < 19; q++) Fl[q] = F[q];
        float rho_s, u1, v1, w1;
        collide_node_pairs<LES>(Fl, sc.rho_mod, sc.f6, sc.f12, sc.tau, sc.lesC, rho_s, u1, v1, w1);
#pragma unroll
        for (int q = 0; q < 19; q++) store_f<S>(fnq[q], (unsigned)node, q, Fl[q]);
        if (macros_on) { rho_out[node] = rho_s; u_out[node] = u1; v_out[node] = v1; w_out[node] = w1; }
        // column partials in FP32 (at most NZ terms), folded into FP64 once per column
        if (y == k.yplane) ub += v1*T.dxf[x]*T.dzf[z];
        mass += rho_s;   // a non-finite density makes the thread's mass sum non-finite (checked once per piece)
    }

    // Copy jobs of a plane (1..18: population q, two pieces when the halo wraps; 19, 20: the
    // target's xi weights and f0 row). Jobs are spread over the four warps (job q on warp q & 3,
    // lane q >> 2) so that no warp serialises all the copy issues; thread 0 posts the expected
    // bytes (a copy may complete before that: the phase cannot end while the arrival is due).
    struct Lane {
        int tid, xl, yl;        // node of this thread within the tile
        // copy job of this lane (lanes 0..5 of warps 0..3: job 4*lane + warp; -1: none)
        int jq, joff;           // population (19, 20: target weights, f0 row), byte offset in its region
        bool jfront, jwide;     // region: front buffer or stage; rows: TY + 6 or TY
    };

    // Copy job of one lane (fixed for the whole kernel, see Lane): population jq of plane p
    // into its region (front buffer or stage s), as TY rows or TY + 6 rows with the streamwise
    // halo (two pieces when the halo wraps); jobs 19 and 20 are the target's xi weights and f0
    // row (only when the plane carries a target). Thread 0 posts the expected bytes first (a
    // copy may complete before that: the phase cannot end while the arrival is due).
    __device__ void issue_plane(unsigned char *smem, int s, uint64_t *bar, int p, int y0, bool tgt, const Lane &L) const {
        constexpr int NX = LY::NX, TY = LY::TY;
        const int NY = k.NY;
        constexpr unsigned row_bytes = (unsigned)(NX*sizeof(S));
        if (L.tid == 0) mbar_expect_tx(bar, LY::pops_bytes() + (tgt ? LY::tgt_bytes : 0u));
        unsigned char *stage = smem + LY::stage_off(s);
        if (L.jq >= 1 && L.jq < 19) {
            S *dst = (S *)((L.jfront ? smem + LY::front_off(s) : stage) + L.joff);
            const S *plane_base = fo + (size_t)L.jq*((size_t)NX*NY*k.NZ) + (size_t)p*NY*NX;
            if (!L.jwide) {
                bulk_g2s(dst, plane_base + (size_t)y0*NX, TY*row_bytes, bar);
            } else {
                const int ys = y0 >= 3 ? y0 - 3 : y0 - 3 + NY;
                constexpr int rows = TY + 6;
                const int first = min(rows, NY - ys);
                bulk_g2s(dst, plane_base + (size_t)ys*NX, first*row_bytes, bar);
                if (first < rows) bulk_g2s(dst + (size_t)first*NX, plane_base, (rows - first)*row_bytes, bar);
            }
        } else if (tgt && L.jq >= 19) {
            if (L.jq == 19) bulk_g2s(stage + LY::w_off, T.wxi + ((size_t)(p - 3)*NY + y0)*64, (unsigned)(TY*64*sizeof(float)), bar);
            if (L.jq == 20) bulk_g2s(stage + LY::f0_off, fo + ((size_t)(p - 3)*NY + y0)*NX, TY*row_bytes, bar);
        }
    }

    // Thread 0, at the end of the kernel: bounded wait for copies still pending (only after a
    // timeout; in a healthy run every copy has been consumed). A wait that runs out here is
    // recorded as a fault too (bit 2), so the host learns of it even when no earlier wait failed.
    __device__ __forceinline__ void drain(unsigned char *smem, unsigned parity, int tid) const {
        if (tid != 0) return;
        uint64_t *bars = (uint64_t *)(smem + LY::bar_off);
        for (int s = 0; s < LY::NS; s++) {
            if (!((parity >> (PEND + s)) & 1u)) continue;
            const unsigned ph = (parity >> (PPAR + s)) & 1u;
            bool done = false;
            for (int it = 0; it < (1 << 22) && !done; ++it) {
                done = mbar_try_wait(&bars[s], ph);
                if (!done && it > 32) __nanosleep(256);
            }
            if (!done) atomicOr(&ctrl->fault, 2u);
        }
    }

    // A piece of a column: targets ta .. tb-1 of tile rows y0 .. y0+TY-1, computed from source
    // planes p0 .. p1 (target t uses planes b(t) .. b(t)+6, see window_base).
    struct Piece {
        int y0, ta, tb, p0, p1;
    };
    // first plane of target t's xi window (the reference's stencil base, clamped at the walls)
    __device__ __forceinline__ int window_base(int t) const {
        return t <= 3 ? 0 : (t >= k.NZ - 4 ? k.NZ - 7 : t - 3);
    }
    // targets 4 .. NZ-4 take their xi weights and f0 row from the stage of plane t + 3
    __device__ __forceinline__ bool staged_target(int p, const Piece &P) const {
        const int t = p - 3;
        return t >= 4 && t <= k.NZ - 4 && t >= P.ta && t < P.tb;
    }

    // After a CTA barrier, lanes 0..5 of every warp start the copies of plane p into stage s;
    // thread 0 (which posts the expected bytes) records the stage as pending. After a timed-out
    // wait anywhere in the CTA (the shared flag, written before the barrier) no copy starts.
    __device__ __forceinline__ void issue(unsigned char *smem, int s, int p, const Piece &P, const Lane &L,
                                          unsigned &parity) const {
        if (L.jq < 0) return;   // lanes 0..5 of warps 0..3 (job 0: thread 0, which only posts the bytes)
        if (*(volatile int *)(smem + LY::flag_off)) return;
        if (p == k.drill_plane) return;   // failure drill: this plane's copies never start
        fence_proxy_async();
        issue_plane(smem, s, (uint64_t *)(smem + LY::bar_off) + s, p, P.y0, staged_target(p, P), L);
        if (L.tid == 0)
            parity = (parity & ~(1u << (PPAR + s))) | (((parity >> s) & 1u) << (PPAR + s)) | (1u << (PEND + s));
    }

    // One source plane (the i-th of its piece): wait for its copies, filter, and store the
    // plane's values in the TMEM ring slot of plane p.
    __device__ __forceinline__ void plane(int i, int p, const Piece &P, unsigned char *smem, unsigned &parity,
                                          bool &faulted, const Lane &L, uint32_t tl, int sp) const {
        constexpr int NX = LY::NX, TY = LY::TY;
        const int s = i % LY::NS;
        uint64_t *bars = (uint64_t *)(smem + LY::bar_off);
        float4 *ybuf = (float4 *)(smem + LY::ybuf_off) + (i & 1)*TY*NX + L.yl*NX;   // this row, this plane
        const S *raw = (const S *)(smem + LY::stage_off(s));   // populations 1, 2, 11..14
        const S *frontp = (const S *)(smem + LY::front_off(s));  // populations read before the barrier
        if (mbar_wait(&bars[s], (parity >> s) & 1u, ctrl, faulted)) parity &= ~(1u << (PEND + s));
        else if (faulted) *(volatile int *)(smem + LY::flag_off) = 1;
        parity ^= 1u << s;
        {   // streamwise filter over rows yl .. yl+6 of the halo copy, and raw values of 5, 6
            const S *base = frontp + L.yl*NX + L.xl;
            auto row = [&](int q, int b) -> const S * { return base + LY::off(q) + b*NX; };
            // packed pairs: the first of each pair departs from y - minSize (weights wy0), the
            // second from y + minSize (wy2)
            P2 a34 = p2(0.f, 0.f), a1516 = a34, a1718 = a34, a79 = a34, a810 = a34;
#pragma unroll
            for (int b = 0; b < 7; b++) {
                const P2 w = p2(tc.wy[b]);
                fma2(a34, w, p2(ldv<S>(row(3, b)), ldv<S>(row(4, b))));
                fma2(a1516, w, p2(ldv<S>(row(15, b)), ldv<S>(row(16, b))));
                fma2(a1718, w, p2(ldv<S>(row(17, b)), ldv<S>(row(18, b))));
                fma2(a79, w, p2(ldv<S>(row(7, b)), ldv<S>(row(9, b))));
                fma2(a810, w, p2(ldv<S>(row(8, b)), ldv<S>(row(10, b))));
            }
            const float2 v34 = unp(a34), v1516 = unp(a1516), v1718 = unp(a1718), v79 = unp(a79), v810 = unp(a810);
            tmem_st8(tl + ring_col(sp), v34.x, v34.y, ldv<S>(row(5, 0)), ldv<S>(row(6, 0)), v1516.x, v1516.y, v1718.x,
                     v1718.y);
            ybuf[L.xl] = make_float4(v79.x, v810.x, v79.y, v810.y);   // 7, 8, 9, 10
        }
        __syncthreads();
        // every thread has finished plane i-1: its stage can take plane p + NS - 1
        if (p + LY::NS - 1 <= P.p1) issue(smem, (i + LY::NS - 1) % LY::NS, p + LY::NS - 1, P, L, parity);
        {   // spanwise filter of this thread's node: x - minSize (wx0) for 7, 9, 1, 11, 13 and
            // x + minSize (wx2) for 8, 10, 2, 12, 14, packed as pairs
            const S *raw_row = raw + L.yl*NX;
            P2 a78 = p2(0.f, 0.f), a910 = a78, a12 = a78, a1112 = a78, a1314 = a78;
#pragma unroll
            for (int a = 0; a < 7; a++) {
                const int xx = wrap_x<NX>(L.xl - 3 + a);
                const P2 w = p2(tc.wx[a]);
                const float4 g = ybuf[xx];
                fma2(a78, w, p2(g.x, g.y));
                fma2(a910, w, p2(g.z, g.w));
                fma2(a12, w, p2(ldv<S>(raw_row + LY::off(1) + xx), ldv<S>(raw_row + LY::off(2) + xx)));
                fma2(a1112, w, p2(ldv<S>(raw_row + LY::off(11) + xx), ldv<S>(raw_row + LY::off(12) + xx)));
                fma2(a1314, w, p2(ldv<S>(raw_row + LY::off(13) + xx), ldv<S>(raw_row + LY::off(14) + xx)));
            }
            const float2 v78 = unp(a78), v910 = unp(a910), v12 = unp(a12), v1112 = unp(a1112), v1314 = unp(a1314);
            tmem_st8(tl + ring_col(sp) + 8, v78.x, v910.x, v78.y, v910.y, v1112.x, v1314.x, v1112.y, v1314.y);
            tmem_st2(tl + r12_col(p), v12.x, v12.y);
        }
    }

    // Target t of tile row y, whose window (planes p-6 .. p) is complete in the ring. Staged
    // targets take their xi weights and f0 row from the stage of plane p; the wall caps read them
    // from global memory.
    __device__ __forceinline__ void target(uint32_t tl, int sp, int t, const unsigned char *stage, int x, int y, int yl,
                                           const Scal &sc, float &ub, float &mass) const {
        constexpr int NX = LY::NX;
        float F[19];
        // window base p - 6 sits in slot (sp + 1) mod 7
        xi_combine(tl, sp == 6 ? 0 : sp + 1, r12_col(t), (const float *)(stage + LY::w_off) + yl*64, F);
        F[0] = ld1<S>((const S *)(stage + LY::f0_off) + yl*NX + x, (float)dev_ref(0));
        finish<false>(F, x, y, t, sc, ub, mass);
    }

    // A wall-cap target (z <= 3 at the window of plane 6, z >= NZ-3 at the window of plane NZ-1):
    // xi weights and f0 from global memory, walls and BFL rows. Out of line, so that the plane
    // loop's code stays small; returns the target's (ub, mass) contributions.
    __device__ __noinline__ float2 cap_target(uint32_t tl, int sp, int t, int x, int y, const Scal &sc) const {
        float F[19];
        xi_combine(tl, sp == 6 ? 0 : sp + 1, r12_col(t), T.wxi + ((size_t)t*k.NY + y)*64, F);
        F[0] = load_f<S>(fo, ((size_t)t*k.NY + y)*LY::NX + x, 0);
        float ub = 0.f, mass = 0.f;
        finish<true>(F, x, y, t, sc, ub, mass);
        return make_float2(ub, mass);
    }

    __device__ __forceinline__ Lane lane() const {
        constexpr int NX = LY::NX;
        Lane L;
        L.tid = threadIdx.x;
        L.xl = L.tid % NX;
        L.yl = L.tid / NX;
        int q = ((L.tid & 31) < 6 && L.tid < 128) ? 4*(L.tid & 31) + (L.tid >> 5) : -1;
        if (q > 20) q = -1;   // jobs 0..20 only
        L.jq = q; L.joff = 0; L.jfront = false; L.jwide = false;
#pragma unroll
        for (int r = 1; r < 19; r++)
            if (q == r) { L.joff = LY::off_bytes(r); L.jfront = LY::front(r); L.jwide = LY::wide(r); }
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

    // One piece of a column: planes P.p0 .. P.p1 through the ring; after plane p the targets
    // whose window ends at p are completed (p = 6: the lower wall cap 0..3; p = NZ-1: targets
    // NZ-4 .. NZ-1; otherwise target p-3). Adds the piece's partial sums to ub and mass.
    __device__ __forceinline__ void piece(const Piece &P, unsigned char *smem, unsigned &parity, bool &faulted,
                                          const Lane &L, uint32_t tl, const Scal &sc, float &ub, float &mass) const {
        const int NZ = k.NZ;
        __syncthreads();   // every thread is done with every stage of the previous piece
        for (int s = 0; s < LY::NS - 1 && P.p0 + s <= P.p1; s++) issue(smem, s, P.p0 + s, P, L, parity);
        const int y = P.y0 + L.yl;
        int sp = P.p0 % 7;   // ring slot of plane p
#pragma unroll 1
        for (int p = P.p0; p <= P.p1; p++, sp = sp == 6 ? 0 : sp + 1) {
            const int i = p - P.p0;
            plane(i, p, P, smem, parity, faulted, L, tl, sp);
            if (i < 6) continue;   // window of plane p not yet in the ring
            const unsigned char *stage = smem + LY::stage_off(i % LY::NS);
            const int lo = p == 6 ? 0 : p - 3, hi = p == NZ - 1 ? NZ - 1 : p - 3;
            for (int t = max(lo, P.ta); t <= min(hi, P.tb - 1); t++) {
                if (t == p - 3 && staged_target(p, P)) {
                    target(tl, sp, t, stage, L.xl, y, L.yl, sc, ub, mass);
                } else {
                    const float2 c = cap_target(tl, sp, t, L.xl, y, sc);
                    ub += c.x;
                    mass += c.y;
                }
            }
        }
    }

    // TMEM ring: warp 0 allocates LY::RING columns; every thread gets the address of its lane
    // (lane quarter w % 4 of warp w) and of its 128-column block (w / 4)
    __device__ __forceinline__ uint32_t ring_alloc(unsigned char *smem, int tid) const {
        uint32_t *slot = (uint32_t *)(smem + LY::flag_off + 8);
        if (tid < 32) {
            tmem_alloc(slot, LY::RING);
            tmem_relinquish();
        }
        tmem_fence_before();
        __syncthreads();
        tmem_fence_after();
        return *(volatile uint32_t *)slot + ((uint32_t)(32*((tid >> 5) & 3)) << 16) + (uint32_t)(128*(tid >> 7));
    }
    __device__ __forceinline__ void ring_free(unsigned char *smem, int tid) const {
        tmem_wait_ld();
        tmem_wait_st();
        tmem_fence_before();
        __syncthreads();
        if (tid < 32) {
            tmem_fence_after();
            tmem_dealloc(*(volatile uint32_t *)(smem + LY::flag_off + 8), LY::RING);
        }
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
        const uint32_t tl = ring_alloc(smem, L.tid);   // includes the CTA barrier after the init
        unsigned parity = 0;   // bit s: parity of the next completion of stage s
        bool faulted = false;
        double ub_total = 0.0, mass_total = 0.0;
        const Scal sc = scalars();
        // Work items: each column is cut into tc.zsegs equal wall-normal segments; item
        // (segment s, tile) = s*ntiles + tile. CTAs take items b, b + G, ..., so the CTAs
        // running at the same time hold neighbouring tiles of the same segment and reach the
        // same plane at about the same time: the streamwise halo rows each CTA copies are the
        // neighbours' own rows, read from HBM once and from L2 by the others.
        const int NZ = k.NZ;
        const int ntiles = k.NY/LY::TY, nseg = tc.zsegs;
        for (int item = blockIdx.x; item < ntiles*nseg; item += gridDim.x) {
            const int tile = item % ntiles, seg = item/ntiles;
            Piece P;
            P.y0 = tile*LY::TY;
            P.ta = seg*NZ/nseg;
            P.tb = (seg + 1)*NZ/nseg;
            P.p0 = window_base(P.ta);
            P.p1 = window_base(P.tb - 1) + 6;
            float ub = 0.f, mass = 0.f;   // this piece's partial sums
            piece(P, smem, parity, faulted, L, tl, sc, ub, mass);
            if (!isfinite(mass)) ctrl->nonfinite = 1u;
            ub_total += (double)ub;
            mass_total += (double)mass;
        }
        drain(smem, parity, L.tid);
        ring_free(smem, L.tid);
        end_of_step<LY::NT>(ctrl, k, tc.n, ub_total, mass_total, true, mass_on != 0,
                              gridDim.x*gridDim.y*gridDim.z);
    }
};

// Batched form: one launch advances every solve of a batch (same storage format and spanwise
// width) by one step. Work items are (solve, segment*ntiles + tile) pairs; a CTA copies the solve's
// descriptor into shared memory, takes the old/new buffers from the solve's own step
// counter (so a graph of identical launches advances the solves step after step), runs the
// piece and reports it to the solve's controller, whose last piece closes the step.
template <class S, bool LES, int NXC>
struct BatchDesc {
    TiledKernel<S, LES, NXC> K;
    S *buf[2];          // population buffers; the old one is buf[step & 1]
    int ntiles;         // tiles of this solve
    int nseg;           // wall-normal segments per column (work items per step: ntiles*nseg)
};

template <class S, bool LES, int NXC>
__global__ void __launch_bounds__(threads_for<NXC>(), 512/threads_for<NXC>())
step_tiled_kernel(TiledKernel<S, LES, NXC> K) { K.run(); }

template <class S, bool LES, int NXC>
__global__ void __launch_bounds__(threads_for<NXC>(), 512/threads_for<NXC>())
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
    const uint32_t tl = K.ring_alloc(smem, tid);   // uses no member of K
    unsigned parity = 0;
    bool faulted = false;
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        const int2 w = items[it];   // (solve, segment*ntiles + tile)
        __syncthreads();            // previous item done with K and every stage
        {
            const unsigned *src = (const unsigned *)&descs[w.x].K;
            unsigned *dst = (unsigned *)kbuf;
            for (int i = tid; i < (int)(sizeof(KT)/4); i += LY::NT) dst[i] = src[i];
        }
        if (tid == 0) step_s = *(volatile unsigned long long *)&descs[w.x].K.ctrl->step;
        __syncthreads();
        if (tid == 0) {
            const unsigned long long st = step_s;
            K.fo = descs[w.x].buf[st & 1ULL];
            K.fn = descs[w.x].buf[(st + 1) & 1ULL];
            const size_t N = (size_t)K.k.NX*K.k.NY*K.k.NZ;
            for (int q = 0; q < 19; q++) K.fnq[q] = K.fn + q*N;
            K.tc.n = st + 1;
            K.mass_on = K.k.mass_interval > 0 && ((st + 1) % (unsigned long long)K.k.mass_interval) == 0ULL;
            K.macros_on = macros_on;
        }
        __syncthreads();
        const auto L = K.lane();
        const auto sc = K.scalars();
        const int nt = descs[w.x].ntiles, ns = descs[w.x].nseg;
        const int tile = w.y % nt, seg = w.y/nt;
        typename KT::Piece P;
        P.y0 = tile*LY::TY;
        P.ta = seg*K.k.NZ/ns;
        P.tb = (seg + 1)*K.k.NZ/ns;
        P.p0 = K.window_base(P.ta);
        P.p1 = K.window_base(P.tb - 1) + 6;
        float ub = 0.f, mass = 0.f;
        K.piece(P, smem, parity, faulted, L, tl, sc, ub, mass);
        if (!isfinite(mass)) K.ctrl->nonfinite = 1u;
        end_of_step<LY::NT>(K.ctrl, K.k, K.tc.n, (double)ub, (double)mass, true, K.mass_on != 0,
                              (unsigned)(nt*ns));
    }
    __syncthreads();
    if (nitems > 0) K.drain(smem, parity, tid);
    K.ring_free(smem, tid);
}

template <class S, bool LES, int NXC>
cudaError_t launch_t(const StepLaunch &L) {
    TiledKernel<S, LES, NXC> K;
    K.fo = (const S *)L.fo;
    K.fn = (S *)L.fn;
    for (int q = 0; q < 19; q++) K.fnq[q] = K.fn + (size_t)q*L.k.NX*L.k.NY*L.k.NZ;
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
    step_tiled_kernel<S, LES, NXC><<<K.tc.grid, Lay<S, NXC>::NT, smem, L.stream>>>(K);
    return cudaGetLastError();
}

template <class S, bool LES>
cudaError_t launch_nx(const StepLaunch &L) {
    switch (L.k.NX) {
    case 32: return launch_t<S, LES, 32>(L);
    case 64: return launch_t<S, LES, 64>(L);
    case 128: return launch_t<S, LES, 128>(L);
    case 256: return launch_t<S, LES, 256>(L);
    case 384: return launch_t<S, LES, 384>(L);
    default: return cudaErrorNotSupported;
    }
}

template <class S>
cudaError_t launch_s(const StepLaunch &L) {
    return L.les ? launch_nx<S, true>(L) : launch_nx<S, false>(L);
}

template <class S> struct LayInfo {
    size_t smem;
    int nt, ctas_per_sm;
};
template <class S, int NXC> LayInfo<S> lay_info() {
    return {(size_t)Lay<S, NXC>::smem_bytes, Lay<S, NXC>::NT, Lay<S, NXC>::CTAS_PER_SM};
}
template <class S>
LayInfo<S> lay_for(int nx) {
    switch (nx) {
    case 32: return lay_info<S, 32>();
    case 64: return lay_info<S, 64>();
    case 128: return lay_info<S, 128>();
    case 256: return lay_info<S, 256>();
    default: return lay_info<S, 384>();
    }
}

}  // namespace

bool tiled_supported(const StepConst &k, int precision) {
    if (precision == ISLBM_FP64) return false;
    // spanwise widths with a compiled layout (tiles of 128 nodes; one row of 256 or 384)
    if (k.NX != 32 && k.NX != 64 && k.NX != 128 && k.NX != 256 && k.NX != 384) return false;
    const int TY = k.NX < 128 ? 128/k.NX : 1;
    if (k.NY % TY != 0 || k.NY < TY + 6 || k.NZ < 8) return false;
    return true;
}

int make_tiled_const(const StepConst &k, int precision, const double *wx0, const double *wx2, const double *wy0,
                     const double *wy2, int num_sms, TiledConst *out) {
    TiledConst tc;
    std::memset(&tc, 0, sizeof(tc));
    tc.TY = k.NX < 128 ? 128/k.NX : 1;
    size_t smem;
    int ctas_tmem;
    if (precision == ISLBM_FP32) { const auto li = lay_for<float>(k.NX); smem = li.smem; ctas_tmem = li.ctas_per_sm; }
    else { const auto li = lay_for<__half>(k.NX); smem = li.smem; ctas_tmem = li.ctas_per_sm; }
    tc.smem_bytes = smem;
    for (int a = 0; a < 7; a++) {
        tc.wx[a] = make_float2((float)wx0[a], (float)wx2[a]);
        tc.wy[a] = make_float2((float)wy0[a], (float)wy2[a]);
    }
    const int tiles = k.NY/tc.TY;
    // persistent CTAs: as many as fit on the SMs by shared memory (228 KB per SM, 1 KB reserved
    // per CTA) and by the TMEM rings (512 columns per SM; also the register bound of the kernel)
    const int per_sm = (int)std::min<size_t>((size_t)ctas_tmem, (228*1024)/(tc.smem_bytes + 1024));
    const int slots = per_sm*num_sms;
    // wall-normal segments per column: enough items to fill the resident slots, each at
    // least 16 targets long (a segment re-reads the 6 planes below it to fill its ring)
    tc.zsegs = std::max(1, std::min(slots/tiles, k.NZ/16));
    tc.grid = std::min(tiles*tc.zsegs, slots);
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
                     void *buf0, void *buf1, int ntiles, int nseg, void *out) {
        D d;
        std::memset((void *)&d, 0, sizeof(d));
        d.K.T = T; d.K.k = k; d.K.tc = tc; d.K.ctrl = ctrl;
        d.K.rho_out = (float *)macros[0]; d.K.u_out = (float *)macros[1];
        d.K.v_out = (float *)macros[2]; d.K.w_out = (float *)macros[3];
        d.buf[0] = (S *)buf0; d.buf[1] = (S *)buf1;
        d.ntiles = ntiles;
        d.nseg = nseg;
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
        step_tiled_batch_kernel<S, LES, NXC><<<grid, Lay<S, NXC>::NT, Lay<S, NXC>::smem_bytes, st>>>((const D *)descs, items,
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
        case 128: return f(BatchOps<S, L, 128>{});
        case 256: return f(BatchOps<S, L, 256>{});
        default: return f(BatchOps<S, L, 384>{});
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
                     Ctrl *ctrl, void *const macros[4], void *buf0, void *buf1, int ntiles, int nseg, void *out) {
    dispatch(precision, NX, les, [&](auto ops) {
        decltype(ops)::fill(T, k, tc, ctrl, macros, buf0, buf1, ntiles, nseg, out);
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
