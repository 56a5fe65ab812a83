// Paired-node tiled step kernel: the tiled step of step_tiled.cu with two spanwise-adjacent
// nodes per thread and every FP32 operation packed across the pair.
//
// Same step as stream_collide (C/evolution.h:358-684) for FP32 arithmetic with FP32, FP16 or
// BF16 population storage. Organisation:
//   * a CTA of 128 threads owns a tile of TY = 256/NX full-width rows (192 threads and one row
//     at NX = 384; two nodes per thread:
//     x0 = 2*(thread % (NX/2)) and x0 + 1) and marches upward through a wall-normal segment of
//     that column; each plane's 18 moving populations are copied global -> shared memory (the
//     ten with e_y != 0 with a 3-row streamwise halo on both sides) as 4D tensor-map boxes
//     (cp.async.bulk.tensor: full rows x halo rows x 2 or 4 consecutive populations per copy;
//     tiles whose halo wraps around the period, and NX = 384, copy row runs with
//     cp.async.bulk). Every operand of a copy is uniform over the CTA, so one thread issues it
//     with a few uniform instructions, but the issuing thread stalls for about 50 cycles per
//     copy: hence few, large copies, the front ones issued by thread 0 and the stage ones by
//     thread 64 (another warp, of the other tile row where a tile has two), so that the two
//     stalls overlap (splitting the front copies as well was slower);
//   * front buffer (populations read before the plane's CTA barrier: the streamwise-filtered
//     ten and the xi-only 5, 6) and stage buffer (1, 2, 11..14, read after it, plus the target
//     row's xi weights and f0) have mbarriers of their own, so the front copies of plane p + 2
//     start as soon as every thread has filtered plane p;
//   * the separable interpolation of step_tiled.cu on node pairs: the streamwise filter reads
//     two nodes per 8-byte shared load; the spanwise filter of 7, 8, 9, 10 reads the
//     streamwise-filtered values of neighbouring nodes (written by their threads as
//     (7, 8, 9, 10) quads) and the spanwise filter of 1, 2, 11..14 reads aligned node pairs and
//     splits each node's sum over the two lanes of a packed accumulator; the xi combination
//     reads a 7-plane ring of filtered node pairs kept in tensor memory (TMEM, 256 columns per
//     128 threads: 7 planes x 16 directions x 2 nodes, plus the F1/F2 delay line) with the xi
//     weights stored as duplicated pairs;
//   * the collision of the pair runs in packed FP32x2 arithmetic (collide_x2), results are
//     stored as node pairs (8-byte stores for FP32, 4-byte for FP16/BF16);
//   * persistent CTAs, two per SM (one at NX = 384; TMEM bound), work items (wall-normal segment, tile) taken
//     segment-major so that CTAs running together share their halo rows through L2.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include <cudaTypedefs.h>

#include "pair_math.cuh"
#include "step_common.cuh"
#include "step_launch.hpp"
#include "step_tiled.hpp"
#include "tile_helpers.cuh"

namespace islbm {

namespace {

template <int NXC> constexpr int pair_threads() { return NXC <= 256 ? 128 : NXC/2; }

// D3Q19 streamwise component of e_q (C/initialization.h:7-12 ordering)
__host__ __device__ constexpr int ey_of(int q) {
    return (q == 3 || q == 7 || q == 8 || q == 15 || q == 17) ? 1 : (q == 4 || q == 9 || q == 10 || q == 16 || q == 18) ? -1 : 0;
}

// populations of the front buffer (the ten streamwise-filtered ones with the halo rows, then
// 5, 6) and of the stage (spanwise-filtered 1, 2, 11..14)
__host__ __device__ constexpr int FQ(int i) {
    return i < 2 ? 3 + i : i < 6 ? 5 + i : i < 10 ? 9 + i : i - 5;   // 3, 4, 7, 8, 9, 10, 15, 16, 17, 18, 5, 6
}
__host__ __device__ constexpr int SQ(int i) { return i < 2 ? 1 + i : 9 + i; }   // 1, 2, 11, 12, 13, 14

// Shared-memory layout of one tile (all offsets compile-time constants).
//   front f (NF of them): FQ(0..9) as TY + 6 rows, FQ(10..11) as TY rows;
//   stage s (NS = 2): SQ as TY rows, the target rows' duplicated xi weights (TY x 128 floats)
//     and the target rows of f0;
//   ybuf [2][TY][NX] float4: streamwise-filtered (7, 8, 9, 10) of every node, by plane parity;
//   mbarriers: NF front, NS stage; then the CTA-wide timeout flag and the TMEM address.
template <class S, int NXC>
struct PLay {
    static constexpr int NX = NXC;
    static constexpr int NT = pair_threads<NXC>();
    static constexpr int PR = NX/2;                  // node pairs per row
    static constexpr int TY = 2*NT/NX;               // rows per tile
    static constexpr int RING = NT <= 128 ? 256 : 512;
    static constexpr int CTAS_PER_SM = 512/RING;     // TMEM bound (512 columns per SM)
    static constexpr int EB = (int)sizeof(S);
    static constexpr int up16(int v) { return (v + 15)/16*16; }
    static constexpr int up128(int v) { return (v + 127)/128*128; }
    static constexpr int frows(int i) { return i < 10 ? TY + 6 : TY; }
    static constexpr int fq_off_bytes(int i) {
        int off = 0;
        for (int r = 0; r < i; r++) off = up16(off + frows(r)*NX*EB);
        return off;
    }
    static constexpr int fq_off(int i) { return fq_off_bytes(i)/EB; }
    static constexpr int front_bytes = up128(fq_off_bytes(12));
    static constexpr unsigned front_tx() {
        unsigned b = 0;
        for (int i = 0; i < 12; i++) b += (unsigned)(frows(i)*NX*EB);
        return b;
    }
    static constexpr int sq_off_bytes(int i) { return i*up16(TY*NX*EB); }
    static constexpr int sq_off(int i) { return sq_off_bytes(i)/EB; }
    static constexpr int w_off = sq_off_bytes(6);                 // within a stage
    static constexpr int f0_off = up16(w_off + TY*128*4);
    static constexpr int stage_bytes = up128(f0_off + TY*NX*EB);
    static constexpr unsigned stage_tx = (unsigned)(6*TY*NX*EB);
    static constexpr unsigned tgt_tx = (unsigned)(TY*128*4 + TY*NX*EB);
    // two front buffers where they fit two CTAs per SM
    static constexpr int NF = (EB == 2 || NX <= 128) ? 2 : 1;
    static constexpr int NS = 2;
    static constexpr int front_off(int f) { return f*front_bytes; }
    static constexpr int stage_off(int s) { return NF*front_bytes + s*stage_bytes; }
    static constexpr int ybuf_off = NF*front_bytes + NS*stage_bytes;
    static constexpr int bar_off = ybuf_off + 2*TY*NX*16;
    static constexpr int flag_off = bar_off + (NF + NS)*8;
    // large enough that no more than CTAS_PER_SM CTAs fit in an SM's 228 KB (1 KB reserved per
    // CTA), so the TMEM allocations of resident CTAs never exceed the SM's 512 columns
    // (a 512-column layout also keeps out a CTA of any 256-column layout, whose floor is 76 KB)
    static constexpr int smem_floor = CTAS_PER_SM == 1 ? 152*1024 : 228*1024/(CTAS_PER_SM + 1) + 1;
    static constexpr int smem_bytes = flag_off + 16 > smem_floor ? flag_off + 16 : smem_floor;
};

// ring columns of a thread's lane: plane slot s (0..6) at 32*s, directions in the order
// RQ = 3, 4, 5, 6, 15, 16, 17, 18 (columns 0..15 of the slot, written after the streamwise
// filter), 7, 8, 9, 10, 11, 12, 13, 14 (columns 16..31, after the spanwise filter), each as
// (node x0, node x0 + 1); the F1/F2 delay line of the last 8 planes at 224 + 4*(p mod 8):
// F1 pair, F2 pair.
__device__ __forceinline__ uint32_t pring_col(int slot) { return 32u*(uint32_t)slot; }
__device__ __forceinline__ uint32_t pdelay_col(int p) { return 224u + 4u*(uint32_t)(p & 7); }

__device__ __forceinline__ void tmem_st16(uint32_t ta, const float (&v)[16]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16};" ::"r"(ta),
        "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7]), "f"(v[8]), "f"(v[9]),
        "f"(v[10]), "f"(v[11]), "f"(v[12]), "f"(v[13]), "f"(v[14]), "f"(v[15])
        : "memory");
}
__device__ __forceinline__ void tmem_st4(uint32_t ta, float a, float b, float c, float d) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1, %2, %3, %4};" ::"r"(ta), "f"(a), "f"(b), "f"(c), "f"(d)
                 : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t ta, uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
          "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
          "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(ta)
        : "memory");
}
__device__ __forceinline__ void tmem_ld4(uint32_t ta, uint32_t (&v)[4]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3])
                 : "r"(ta)
                 : "memory");
}

// two stored values of adjacent nodes -> FP32 pair (the deviation formats give deviations)
template <class S> __device__ __forceinline__ V2 ld2v(const S *p);
template <> __device__ __forceinline__ V2 ld2v<float>(const float *p) { return V2(*(const float2 *)p); }
template <> __device__ __forceinline__ V2 ld2v<__half>(const __half *p) { return V2(__half22float2(*(const __half2 *)p)); }
template <> __device__ __forceinline__ V2 ld2v<__nv_bfloat16>(const __nv_bfloat16 *p) {
    return V2(__bfloat1622float2(*(const __nv_bfloat162 *)p));
}
// full values of a node pair from global memory (read-only path)
template <class S> __device__ __forceinline__ V2 ld2g(const S *p, int q) {
    V2 v;
    if constexpr (std::is_same<S, float>::value) v = V2(__ldg((const float2 *)p));
    else if constexpr (std::is_same<S, __half>::value) {
        const unsigned r = __ldg((const unsigned *)p);
        v = V2(__half22float2(*(const __half2 *)&r));
    } else {
        const unsigned r = __ldg((const unsigned *)p);
        v = V2(__bfloat1622float2(*(const __nv_bfloat162 *)&r));
    }
    if constexpr (Storage<S>::dev) v = v + V2((float)dev_ref(q));
    return v;
}
// store a node pair (full values; the deviation formats store f - ref)
template <class S> __device__ __forceinline__ void st2(S *p, V2 v, int q) {
    if constexpr (std::is_same<S, float>::value) *(float2 *)p = v.v;
    else {
        const V2 d = v - V2((float)dev_ref(q));
        if constexpr (std::is_same<S, __half>::value) *(__half2 *)p = __float22half2_rn(d.v);
        else *(__nv_bfloat162 *)p = __float22bfloat162_rn(d.v);
    }
}

// Tensor copy of one box (x, y, z, q) of a population buffer: the box lands in shared memory as
// [q][rows][NX], the layout of the front and stage buffers.
__device__ __forceinline__ void tma_load4(void *dst, const CUtensorMap *map, int x, int y, int z, int q, uint64_t *bar) {
    asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];"
                 ::"r"(smem_u32(dst)), "l"((unsigned long long)map), "r"(x), "r"(y), "r"(z), "r"(q), "r"(smem_u32(bar))
                 : "memory");
}

// The four tensor maps of the buffer a launch reads (kernel parameter: tensor maps must live in
// parameter, constant or global memory)
struct PairTM {
    CUtensorMap m[4];
};

template <int NX> __device__ __forceinline__ int pwrap(int v) {
    if constexpr ((NX & (NX - 1)) == 0) return v & (NX - 1);
    else return v < 0 ? v + NX : (v >= NX ? v - NX : v);
}

template <class S, bool LES, int NXC>
struct PairKernel {
    using LY = PLay<S, NXC>;
    struct Scal { float f6, f12, rho_mod, tau, lesC; };
    const S *__restrict__ fo;
    S *__restrict__ fn;
    S *fnq[19];                // fn + q*N
    Tables<float> T;
    StepConst k;
    TiledConst tc;
    Ctrl *ctrl;
    float *rho_out, *u_out, *v_out, *w_out;
    int macros_on, mass_on;

    struct Lane {
        int tid, yl, x0;
        uint32_t tl;           // TMEM address of this warp's lane quarter and column block
    };
    struct Piece {
        int y0, ta, tb, p0, p1;
    };
    // pipeline word (every thread): bits 0..1 front parities, 2..3 stage parities; the issuing
    // threads also keep bits 8.. (pending copies of front f / stage s) and 16.. (their parities)
    static constexpr int FP = 0, SP = 2, PENDF = 8, PENDS = 10, PPARF = 16, PPARS = 18;

    // Walls, BFL rows, collision and stores of the node pair (x0, x0 + 1) at row y, plane z,
    // whose streamed populations are in F (F[1..18] filtered values, deviations for the
    // deviation formats; F[0] full). CAP: a wall-cap target, the only ones that can be wall
    // rows (bounce-back at z = 0 and NZ-1, BFL rows at z <= 1).
    template <bool CAP>
    __device__ __forceinline__ void finish(V2 (&F)[19], int x0, int y, int z, const Scal &sc, float &ub, V2 &mass) const {
        constexpr int NX = LY::NX;
        const int NY = k.NY;
        const size_t N = (size_t)NX*NY*k.NZ;
        const unsigned node = (unsigned)(((size_t)z*NY + y)*NX + x0);
        if constexpr (Storage<S>::dev) {
#pragma unroll
            for (int q = 1; q < 19; q++) F[q] = F[q] + V2((float)dev_ref(q));
        }
        if (CAP && z == 0) {
            const S *b = fo + node;
            F[5] = ld2g<S>(b + 6*N, 6); F[11] = ld2g<S>(b + 14*N, 14); F[12] = ld2g<S>(b + 13*N, 13);
            F[15] = ld2g<S>(b + 18*N, 18); F[16] = ld2g<S>(b + 17*N, 17);
        }
        if (CAP && z == k.NZ - 1) {
            const S *b = fo + node;
            F[6] = ld2g<S>(b + 5*N, 5); F[13] = ld2g<S>(b + 12*N, 12); F[14] = ld2g<S>(b + 11*N, 11);
            F[17] = ld2g<S>(b + 16*N, 16); F[18] = ld2g<S>(b + 15*N, 15);
        }
        if (CAP && z <= 1) {
            const int nb = 2*k.NYD6, r = z*k.NYD6 + (y + 3);
            if (T.bfl_flag[r] | T.bfl_flag[nb + r] | T.bfl_flag[2*nb + r] | T.bfl_flag[3*nb + r]) {
                // the out-of-line BFL rows work on per-node copies
                float G0[19], G1[19];
#pragma unroll
                for (int q = 0; q < 19; q++) { G0[q] = F[q].v.x; G1[q] = F[q].v.y; }
                bfl_node<S>(fo, T, k, x0, y, z, G0);
                bfl_node<S>(fo, T, k, x0 + 1, y, z, G1);
#pragma unroll
                for (int q = 0; q < 19; q++) F[q] = V2(G0[q], G1[q]);
            }
        }
        V2 rho, u1, v1, w1;
        collide_x2<LES>(F, sc.rho_mod, sc.f6, sc.f12, sc.tau, sc.lesC, rho, u1, v1, w1);
#pragma unroll
        for (int q = 0; q < 19; q++) st2<S>(fnq[q] + node, F[q], q);
        if (macros_on) {
            *(float2 *)(rho_out + node) = rho.v; *(float2 *)(u_out + node) = u1.v;
            *(float2 *)(v_out + node) = v1.v; *(float2 *)(w_out + node) = w1.v;
        }
        // column partials in FP32 (at most NZ terms), folded into FP64 once per piece
        if (y == k.yplane) ub += (v1.v.x*T.dxf[x0] + v1.v.y*T.dxf[x0 + 1])*T.dzf[z];
        mass = mass + rho;   // a non-finite density makes the mass sum non-finite (checked once per piece)
    }

    // Copies of plane p: the front part into front buffer f and/or the stage part (with the target
    // rows of plane p - 3 when that target is staged) into stage s. Called by every thread after a
    // CTA barrier; thread FRONT_ISSUER issues the front copies and STAGE_ISSUER the stage copies
    // (their operands are uniform over the CTA), each posting its buffer's expected bytes first and
    // keeping the buffer's pending record for the drain.
    static constexpr int FRONT_ISSUER = 0, STAGE_ISSUER = 64;
    // tm: the buffer's tensor maps (box 0: 3, 4 and box 1: 7..10 / 15..18 over the TY + 6 rows;
    // box 2: 5, 6 / 1, 2 and box 3: 11..14 over the TY rows), one copy per box; tiles whose halo
    // wraps around the streamwise period, and launches without maps, copy row runs instead.
    __device__ __forceinline__ void issue(unsigned char *smem, int p, int f, int s, bool do_front, bool do_stage,
                                          const Piece &P, unsigned &pipe, int tid, const CUtensorMap *tm) const {
        constexpr int NX = LY::NX, TY = LY::TY;
        do_front = do_front && tid == FRONT_ISSUER;
        do_stage = do_stage && tid == STAGE_ISSUER;
        if (!do_front && !do_stage) return;
        if (*(volatile int *)(smem + LY::flag_off)) return;   // a wait timed out: no further copies
        if (p == k.drill_plane) return;                        // failure drill: this plane never arrives
        const int NY = k.NY;
        const size_t N = (size_t)NX*NY*k.NZ;
        constexpr unsigned row_bytes = (unsigned)(NX*sizeof(S));
        uint64_t *bars = (uint64_t *)(smem + LY::bar_off);
        const S *plane = fo + (size_t)p*NY*NX;
        fence_proxy_async();
        if (do_front) {
            uint64_t *bar = bars + f;
            mbar_expect_tx(bar, LY::front_tx());
            pipe = (pipe & ~(1u << (PPARF + f))) | (((pipe >> (FP + f)) & 1u) << (PPARF + f)) | (1u << (PENDF + f));
            unsigned char *dst = smem + LY::front_off(f);
            constexpr int rows = TY + 6;
            if (tm && P.y0 >= 3 && P.y0 + TY + 3 <= NY) {
                tma_load4(dst + LY::fq_off_bytes(0), tm + 0, 0, P.y0 - 3, p, 3, bar);
                tma_load4(dst + LY::fq_off_bytes(2), tm + 1, 0, P.y0 - 3, p, 7, bar);
                tma_load4(dst + LY::fq_off_bytes(6), tm + 1, 0, P.y0 - 3, p, 15, bar);
                tma_load4(dst + LY::fq_off_bytes(10), tm + 2, 0, P.y0, p, 5, bar);
            } else {
                const int ys = P.y0 >= 3 ? P.y0 - 3 : P.y0 - 3 + NY;
                const int first = min(rows, NY - ys);
#pragma unroll
                for (int i = 0; i < 10; i++) {
                    S *d = (S *)(dst + LY::fq_off_bytes(i));
                    const S *src = plane + (size_t)FQ(i)*N;
                    bulk_g2s(d, src + (size_t)ys*NX, first*row_bytes, bar);
                    if (first < rows) bulk_g2s(d + (size_t)first*NX, src, (rows - first)*row_bytes, bar);
                }
#pragma unroll
                for (int i = 10; i < 12; i++)
                    bulk_g2s(dst + LY::fq_off_bytes(i), plane + (size_t)FQ(i)*N + (size_t)P.y0*NX, TY*row_bytes, bar);
            }
        }
        if (do_stage) {
            uint64_t *bar = bars + LY::NF + s;
            const int t = p - 3;
            const bool tgt = t >= 4 && t <= k.NZ - 4 && t >= P.ta && t < P.tb;
            mbar_expect_tx(bar, LY::stage_tx + (tgt ? LY::tgt_tx : 0u));
            pipe = (pipe & ~(1u << (PPARS + s))) | (((pipe >> (SP + s)) & 1u) << (PPARS + s)) | (1u << (PENDS + s));
            unsigned char *dst = smem + LY::stage_off(s);
            if (tm) {
                tma_load4(dst + LY::sq_off_bytes(0), tm + 2, 0, P.y0, p, 1, bar);
                tma_load4(dst + LY::sq_off_bytes(2), tm + 3, 0, P.y0, p, 11, bar);
            } else {
#pragma unroll
                for (int i = 0; i < 6; i++)
                    bulk_g2s(dst + LY::sq_off_bytes(i), plane + (size_t)SQ(i)*N + (size_t)P.y0*NX, TY*row_bytes, bar);
            }
            if (tgt) {
                bulk_g2s(dst + LY::w_off, T.wxi2 + ((size_t)t*NY + P.y0)*128, (unsigned)(TY*128*sizeof(float)), bar);
                bulk_g2s(dst + LY::f0_off, fo + ((size_t)t*NY + P.y0)*NX, TY*row_bytes, bar);
            }
        }
    }

    // The issuing threads, at the end of the kernel: bounded wait for the copies they issued that
    // are still pending (only after a timeout; in a healthy run every copy has been consumed). A
    // wait that runs out here is recorded as a fault too.
    __device__ __forceinline__ void drain(unsigned char *smem, unsigned pipe, int tid) const {
        if (tid != FRONT_ISSUER && tid != STAGE_ISSUER) return;
        uint64_t *bars = (uint64_t *)(smem + LY::bar_off);
        for (int b = 0; b < LY::NF + LY::NS; b++) {
            const bool front = b < LY::NF;
            if (tid != (front ? FRONT_ISSUER : STAGE_ISSUER)) continue;
            const int i = front ? b : b - LY::NF;
            if (!((pipe >> ((front ? PENDF : PENDS) + i)) & 1u)) continue;
            const unsigned ph = (pipe >> ((front ? PPARF : PPARS) + i)) & 1u;
            bool done = false;
            for (int it = 0; it < (1 << 22) && !done; ++it) {
                done = mbar_try_wait(&bars[b], ph);
                if (!done && it > 32) __nanosleep(256);
            }
            if (!done) atomicOr(&ctrl->fault, 2u);
        }
    }

    __device__ __forceinline__ int window_base(int t) const {
        return t <= 3 ? 0 : (t >= k.NZ - 4 ? k.NZ - 7 : t - 3);
    }
    __device__ __forceinline__ bool staged_target(int p, const Piece &P) const {
        const int t = p - 3;
        return t >= 4 && t <= k.NZ - 4 && t >= P.ta && t < P.tb;
    }

    // wait for a completion of mbarrier b (front f = b, stage s = NF + s); on a timeout the
    // CTA-wide flag stops further copies
    __device__ __forceinline__ void wait_bar(unsigned char *smem, int b, int pbit, unsigned &pipe, bool &faulted,
                                             int pend_bit, int tid) const {
        uint64_t *bars = (uint64_t *)(smem + LY::bar_off);
        if (mbar_wait(&bars[b], (pipe >> pbit) & 1u, ctrl, faulted)) {
            pipe &= ~(1u << pend_bit);   // (meaningful in the issuer's word only)
        } else if (faulted) {
            *(volatile int *)(smem + LY::flag_off) = 1;
        }
        pipe ^= 1u << pbit;
    }

    // One source plane (the i-th of its piece): filter, store the plane's values in ring slot sp.
    __device__ __forceinline__ void plane(int i, int p, const Piece &P, unsigned char *smem, unsigned &pipe,
                                          bool &faulted, const Lane &L, int sp, const CUtensorMap *tm) const {
        constexpr int NX = LY::NX;
        const int f = LY::NF == 2 ? (i & 1) : 0, s = i & 1;
        wait_bar(smem, f, FP + f, pipe, faulted, PENDF + f, L.tid);
        float4 *yb = (float4 *)(smem + LY::ybuf_off) + (i & 1)*LY::TY*NX + L.yl*NX;
        {   // streamwise filter of the ten over the halo rows yl .. yl+6; raw 5, 6
            const S *base = (const S *)(smem + LY::front_off(f)) + L.yl*NX + L.x0;
            V2 acc[10];
#pragma unroll
            for (int j = 0; j < 10; j++) acc[j] = V2(0.f);
#pragma unroll
            for (int b = 0; b < 7; b++) {
                const V2 w0 = V2(tc.wyb[0][b]), w2 = V2(tc.wyb[1][b]);
#pragma unroll
                for (int j = 0; j < 10; j++) acc[j] = (ey_of(FQ(j)) > 0 ? w0 : w2)*ld2v<S>(base + LY::fq_off(j) + b*NX) + acc[j];
            }
            const V2 r5 = ld2v<S>(base + LY::fq_off(10)), r6 = ld2v<S>(base + LY::fq_off(11));
            // ring columns 0..15: 3, 4, 5, 6, 15, 16, 17, 18 (FQ index 0, 1, -, -, 6, 7, 8, 9)
            const float v[16] = {acc[0].v.x, acc[0].v.y, acc[1].v.x, acc[1].v.y, r5.v.x, r5.v.y, r6.v.x, r6.v.y,
                                 acc[6].v.x, acc[6].v.y, acc[7].v.x, acc[7].v.y, acc[8].v.x, acc[8].v.y, acc[9].v.x, acc[9].v.y};
            tmem_st16(L.tl + pring_col(sp), v);
            // (7, 8, 9, 10) = FQ index 2, 3, 4, 5
            yb[L.x0] = make_float4(acc[2].v.x, acc[3].v.x, acc[4].v.x, acc[5].v.x);
            yb[L.x0 + 1] = make_float4(acc[2].v.y, acc[3].v.y, acc[4].v.y, acc[5].v.y);
        }
        __syncthreads();
        // every thread has filtered plane p (front f free) and finished plane p-1 (stage s^1 free)
        if (LY::NF == 2) {
            if (p + 2 <= P.p1) issue(smem, p + 2, f, 0, true, false, P, pipe, L.tid, tm);
            if (p + 1 <= P.p1) issue(smem, p + 1, 0, s ^ 1, false, true, P, pipe, L.tid, tm);
        } else if (p + 1 <= P.p1) {
            issue(smem, p + 1, 0, s ^ 1, true, true, P, pipe, L.tid, tm);
        }
        wait_bar(smem, LY::NF + s, SP + s, pipe, faulted, PENDS + s, L.tid);
        {   // spanwise filters
            const float4 *g = (const float4 *)(smem + LY::ybuf_off) + (i & 1)*LY::TY*NX + L.yl*NX;
            float4 gv[8];
#pragma unroll
            for (int a = 0; a < 8; a++) gv[a] = g[pwrap<NX>(L.x0 - 3 + a)];
            V2 n0a = V2(0.f), n0b = n0a, n1a = n0a, n1b = n0a;   // (7, 8) and (9, 10) of node 0 / node 1
#pragma unroll
            for (int a = 0; a < 7; a++) {
                const V2 w = V2(tc.wx[a]);
                n0a = w*V2(gv[a].x, gv[a].y) + n0a;
                n0b = w*V2(gv[a].z, gv[a].w) + n0b;
                n1a = w*V2(gv[a + 1].x, gv[a + 1].y) + n1a;
                n1b = w*V2(gv[a + 1].z, gv[a + 1].w) + n1b;
            }
            // 1, 2, 11..14 from aligned node pairs L[k] = (v[x0+k], v[x0+k+1]), k = -4, -2, .., 4: node 0
            // sums w[k+3] v[x0+k] + w[k+4] v[x0+k+1], node 1 w[k+2] v[x0+k] + w[k+3] v[x0+k+1], each
            // split over the two lanes of its accumulator (odd and even stencil points). The two
            // single-lane end terms are separate products, so that no zero weight multiplies a
            // value outside a node's stencil, and both nodes add the same terms in the same order.
            const S *row = (const S *)(smem + LY::stage_off(s)) + L.yl*NX;
            int xo[5];
#pragma unroll
            for (int kk = 0; kk < 5; kk++) xo[kk] = pwrap<NX>(L.x0 - 4 + 2*kk);
            float out[6][2];
#pragma unroll
            for (int r = 0; r < 6; r++) {
                const int set = (SQ(r) == 1 || SQ(r) == 11 || SQ(r) == 13) ? 0 : 1;   // x - minSize : x + minSize
                V2 Lk[5];
#pragma unroll
                for (int kk = 0; kk < 5; kk++) Lk[kk] = ld2v<S>(row + LY::sq_off(r) + xo[kk]);
                V2 a0 = V2(0.f, tc.wxa[set][0].y*Lk[0].v.y), a1 = V2(tc.wxb[set][0])*Lk[1];
#pragma unroll
                for (int kk = 1; kk < 4; kk++) {
                    a0 = V2(tc.wxa[set][kk])*Lk[kk] + a0;
                    if (kk < 3) a1 = V2(tc.wxb[set][kk])*Lk[kk + 1] + a1;
                }
                a1.v.x = __fmaf_rn(tc.wxb[set][3].x, Lk[4].v.x, a1.v.x);
                out[r][0] = a0.v.x + a0.v.y;
                out[r][1] = a1.v.x + a1.v.y;
            }
            const float n0a_x = n0a.v.x, n0a_y = n0a.v.y, n0b_x = n0b.v.x, n0b_y = n0b.v.y;
            const float v[16] = {n0a_x, n1a.v.x, n0a_y, n1a.v.y, n0b_x, n1b.v.x, n0b_y, n1b.v.y,
                                 out[2][0], out[2][1], out[3][0], out[3][1], out[4][0], out[4][1], out[5][0], out[5][1]};
            tmem_st16(L.tl + pring_col(sp) + 16, v);
            tmem_st4(L.tl + pdelay_col(p), out[0][0], out[0][1], out[1][0], out[1][1]);
        }
    }

    // xi combination of the window of planes b .. b+6 held in the ring (sb = b mod 7), with the
    // duplicated-pair xi weights of the target row w (7 x 16 floats: (xi3, xi3, xi4, xi4, xi5,
    // xi5, xi6, xi6, xi15, xi15, ..., xi18, xi18) per stencil point). Writes F[1..18].
    template <class WP>
    __device__ __forceinline__ void xi_combine(uint32_t tl, int sb, int t, WP w, V2 (&F)[19]) const {
        V2 acc[16];
#pragma unroll
        for (int j = 0; j < 16; j++) acc[j] = V2(0.f);
        auto add = [&](const uint32_t (&g)[32], int c) {
            float4 wq[4];
#pragma unroll
            for (int m = 0; m < 4; m++) wq[m] = w(c, m);
            const V2 x3(wq[0].x, wq[0].y), x4(wq[0].z, wq[0].w), x5(wq[1].x, wq[1].y), x6(wq[1].z, wq[1].w);
            const V2 x15(wq[2].x, wq[2].y), x16(wq[2].z, wq[2].w), x17(wq[3].x, wq[3].y), x18(wq[3].z, wq[3].w);
            auto G = [&](int j) { return V2(__uint_as_float(g[2*j]), __uint_as_float(g[2*j + 1])); };
            // slot order 3, 4, 5, 6, 15, 16, 17, 18, 7, 8, 9, 10, 11, 12, 13, 14
            const V2 wj[16] = {x3, x4, x5, x6, x15, x16, x17, x18, x3, x3, x4, x4, x5, x5, x6, x6};
#pragma unroll
            for (int j = 0; j < 16; j++) acc[j] = wj[j]*G(j) + acc[j];
        };
        int s = sb;
#pragma unroll
        for (int c = 0; c < 6; c += 2) {
            uint32_t g0[32], g1[32];
            const int s1 = s == 6 ? 0 : s + 1;
            tmem_ld32(tl + pring_col(s), g0);
            tmem_ld32(tl + pring_col(s1), g1);
            tmem_wait_ld();
            tmem_tie(g0);
            tmem_tie(g1);
            add(g0, c);
            add(g1, c + 1);
            s = s1 == 6 ? 0 : s1 + 1;
        }
        {
            uint32_t g0[32], r[4];
            tmem_wait_st();   // the newest plane's ring stores were issued by this thread just before
            tmem_ld32(tl + pring_col(s), g0);
            tmem_ld4(tl + pdelay_col(t), r);
            tmem_wait_ld();
            tmem_tie(g0);
            tmem_tie(r);
            add(g0, 6);
            F[1] = V2(__uint_as_float(r[0]), __uint_as_float(r[1]));
            F[2] = V2(__uint_as_float(r[2]), __uint_as_float(r[3]));
        }
        constexpr int RQ[16] = {3, 4, 5, 6, 15, 16, 17, 18, 7, 8, 9, 10, 11, 12, 13, 14};
#pragma unroll
        for (int j = 0; j < 16; j++) F[RQ[j]] = acc[j];
    }

    // staged target t of tile row y: weights and f0 from the stage of plane t + 3
    __device__ __forceinline__ void target(const Lane &L, int sp, int t, const unsigned char *stage, int y,
                                           const Scal &sc, float &ub, V2 &mass) const {
        constexpr int NX = LY::NX;
        V2 F[19];
        const float4 *wrow = (const float4 *)(stage + LY::w_off) + L.yl*32;
        xi_combine(L.tl, sp == 6 ? 0 : sp + 1, t, [&](int c, int m) { return wrow[4*c + m]; }, F);
        F[0] = ld2v<S>((const S *)(stage + LY::f0_off) + L.yl*NX + L.x0);
        if constexpr (Storage<S>::dev) F[0] = F[0] + V2((float)dev_ref(0));
        finish<false>(F, L.x0, y, t, sc, ub, mass);
    }

    // wall-cap target (z <= 3 at plane 6, z >= NZ-4 at plane NZ-1): weights and f0 from global
    // memory, walls and BFL rows; out of line. Returns (ub, mass) contributions.
    __device__ __noinline__ float3 cap_target(const Lane &L, int sp, int t, int y, const Scal &sc) const {
        V2 F[19];
        const float4 *wrow = (const float4 *)(T.wxi2 + ((size_t)t*k.NY + y)*128);
        xi_combine(L.tl, sp == 6 ? 0 : sp + 1, t, [&](int c, int m) { return __ldg(wrow + 4*c + m); }, F);
        F[0] = ld2g<S>(fo + ((size_t)t*k.NY + y)*LY::NX + L.x0, 0);
        float ub = 0.f;
        V2 mass = V2(0.f);
        finish<true>(F, L.x0, y, t, sc, ub, mass);
        return make_float3(ub, mass.v.x, mass.v.y);
    }

    __device__ __forceinline__ Lane lane(uint32_t tbase) const {
        Lane L;
        L.tid = threadIdx.x;
        L.yl = L.tid/LY::PR;
        L.x0 = 2*(L.tid % LY::PR);
        const int warp = __shfl_sync(0xffffffffu, L.tid >> 5, 0);
        L.tl = tbase + ((uint32_t)(32*(warp & 3)) << 16) + (uint32_t)(256*(warp >> 2));
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

    __device__ __forceinline__ void piece(const Piece &P, unsigned char *smem, unsigned &pipe, bool &faulted,
                                          const Lane &L, const Scal &sc, float &ub, V2 &mass, const CUtensorMap *tm) const {
        const int NZ = k.NZ;
        __syncthreads();   // every thread is done with every buffer of the previous piece
        issue(smem, P.p0, 0, 0, true, true, P, pipe, L.tid, tm);
        if (LY::NF == 2 && P.p0 + 1 <= P.p1) issue(smem, P.p0 + 1, 1, 0, true, false, P, pipe, L.tid, tm);
        const int y = P.y0 + L.yl;
        int sp = P.p0 % 7;
#pragma unroll 1
        for (int p = P.p0; p <= P.p1; p++, sp = sp == 6 ? 0 : sp + 1) {
            const int i = p - P.p0;
            plane(i, p, P, smem, pipe, faulted, L, sp, tm);
            if (i < 6) {
                // the ring slots a target reads first must be complete: the newest plane's are
                // waited for inside xi_combine, every older one by then
                if (i == 5) tmem_wait_st();
                continue;
            }
            const unsigned char *stage = smem + LY::stage_off(i & 1);
            const int lo = p == 6 ? 0 : p - 3, hi = p == NZ - 1 ? NZ - 1 : p - 3;
            for (int t = max(lo, P.ta); t <= min(hi, P.tb - 1); t++) {
                if (t == p - 3 && staged_target(p, P)) {
                    target(L, sp, t, stage, y, sc, ub, mass);
                } else {
                    const float3 c = cap_target(L, sp, t, y, sc);
                    ub += c.x;
                    mass = mass + V2(c.y, c.z);
                }
            }
        }
    }

    __device__ __forceinline__ uint32_t ring_alloc(unsigned char *smem, int tid) const {
        uint32_t *slot = (uint32_t *)(smem + LY::flag_off + 8);
        if (tid < 32) {
            tmem_alloc(slot, LY::RING);
            tmem_relinquish();
        }
        tmem_fence_before();
        __syncthreads();
        tmem_fence_after();
        return *(volatile uint32_t *)slot;
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

    __device__ void init_bars(unsigned char *smem, int tid) const {
        if (tid == 0) {
            uint64_t *bars = (uint64_t *)(smem + LY::bar_off);
            for (int b = 0; b < LY::NF + LY::NS; b++) mbar_init(&bars[b], 1);
            *(volatile int *)(smem + LY::flag_off) = 0;
            fence_mbar_init();
        }
    }

    __device__ void run(const CUtensorMap *tm) const {
        extern __shared__ __align__(128) unsigned char smem[];
        if (smem_u32(smem) & 127u) tm = nullptr;   // tensor copies need 128-byte aligned destinations
        init_bars(smem, threadIdx.x);
        const Lane L = lane(ring_alloc(smem, threadIdx.x));   // ring_alloc includes the CTA barrier after the init
        unsigned pipe = 0;
        bool faulted = false;
        double ub_total = 0.0, mass_total = 0.0;
        const Scal sc = scalars();
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
            float ub = 0.f;
            V2 mass = V2(0.f);
            piece(P, smem, pipe, faulted, L, sc, ub, mass, tm);
            const float m = mass.v.x + mass.v.y;
            if (!isfinite(m)) ctrl->nonfinite = 1u;
            ub_total += (double)ub;
            mass_total += (double)m;
        }
        drain(smem, pipe, L.tid);
        ring_free(smem, L.tid);
        end_of_step<LY::NT>(ctrl, k, tc.n, ub_total, mass_total, true, mass_on != 0, gridDim.x*gridDim.y*gridDim.z);
    }
};

template <class S, bool LES, int NXC>
struct PairBatchDesc {
    CUtensorMap tm[2][4];   // tensor maps of buf[0], buf[1] (used when tm_on)
    PairKernel<S, LES, NXC> K;
    S *buf[2];          // population buffers; the old one is buf[step & 1]
    int ntiles;
    int nseg;
    int tm_on;
};

template <class S, bool LES, int NXC>
__global__ void __launch_bounds__(pair_threads<NXC>(), 512/PLay<S, NXC>::RING)
step_pair_kernel(const __grid_constant__ PairKernel<S, LES, NXC> K, const __grid_constant__ PairTM T, int tm_on) {
    K.run(tm_on ? T.m : nullptr);
}

// Batched form (serving): work items (solve, segment*ntiles + tile) of many solves of the same
// storage format and width; each CTA copies the item's solve descriptor into shared memory and
// takes the buffers from the solve's own step counter (a graph of identical launches advances
// every solve step after step).
template <class S, bool LES, int NXC>
__global__ void __launch_bounds__(pair_threads<NXC>(), 512/PLay<S, NXC>::RING)
step_pair_batch_kernel(const PairBatchDesc<S, LES, NXC> *__restrict__ descs, const int2 *__restrict__ items, int nitems,
                       int macros_on) {
    using KT = PairKernel<S, LES, NXC>;
    using LY = PLay<S, NXC>;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(16) unsigned char kbuf[sizeof(KT)];
    __shared__ unsigned long long step_s;
    KT &K = *(KT *)kbuf;
    const int tid = threadIdx.x;
    K.init_bars(smem, tid);
    const auto L = K.lane(K.ring_alloc(smem, tid));   // neither uses a member of K
    unsigned pipe = 0;
    bool faulted = false;
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        const int2 w = items[it];
        __syncthreads();            // previous item done with K and every buffer
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
        const auto sc = K.scalars();
        const int nt = descs[w.x].ntiles, ns = descs[w.x].nseg;
        const int tile = w.y % nt, seg = w.y/nt;
        typename KT::Piece P;
        P.y0 = tile*LY::TY;
        P.ta = seg*K.k.NZ/ns;
        P.tb = (seg + 1)*K.k.NZ/ns;
        P.p0 = K.window_base(P.ta);
        P.p1 = K.window_base(P.tb - 1) + 6;
        float ub = 0.f;
        V2 mass = V2(0.f);
        const CUtensorMap *tm = descs[w.x].tm_on && !(smem_u32(smem) & 127u) ? descs[w.x].tm[step_s & 1ULL] : nullptr;
        K.piece(P, smem, pipe, faulted, L, sc, ub, mass, tm);
        const float m = mass.v.x + mass.v.y;
        if (!isfinite(m)) K.ctrl->nonfinite = 1u;
        end_of_step<LY::NT>(K.ctrl, K.k, K.tc.n, (double)ub, (double)m, true, K.mass_on != 0, (unsigned)(nt*ns));
    }
    __syncthreads();
    if (nitems > 0) K.drain(smem, pipe, tid);
    K.ring_free(smem, tid);
}

template <class S, bool LES, int NXC>
cudaError_t launch_p(const StepLaunch &L) {
    PairKernel<S, LES, NXC> K;
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
    PairTM T;
    std::memset((void *)&T, 0, sizeof(T));
    if (L.pmaps) std::memcpy((void *)T.m, L.pmaps, sizeof(T.m));
    static bool attr_done = false;   // one attribute call per instantiation
    constexpr size_t smem = PLay<S, NXC>::smem_bytes;
    if (!attr_done) {
        cudaError_t e = cudaFuncSetAttribute(step_pair_kernel<S, LES, NXC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr_done = true;
    }
    step_pair_kernel<S, LES, NXC><<<K.tc.grid, PLay<S, NXC>::NT, smem, L.stream>>>(K, T, L.pmaps != nullptr);
    return cudaGetLastError();
}

template <class S, bool LES>
cudaError_t launch_pnx(const StepLaunch &L) {
    switch (L.k.NX) {
    case 32: return launch_p<S, LES, 32>(L);
    case 64: return launch_p<S, LES, 64>(L);
    case 128: return launch_p<S, LES, 128>(L);
    case 256: return launch_p<S, LES, 256>(L);
    case 384: return launch_p<S, LES, 384>(L);
    default: return cudaErrorNotSupported;
    }
}

struct PLayInfo {
    size_t smem;
    int nt, ctas_per_sm, ty;
};
template <class S, int NXC> PLayInfo play_info() {
    return {(size_t)PLay<S, NXC>::smem_bytes, PLay<S, NXC>::NT, PLay<S, NXC>::CTAS_PER_SM, PLay<S, NXC>::TY};
}
template <class S> PLayInfo play_for(int nx) {
    switch (nx) {
    case 32: return play_info<S, 32>();
    case 64: return play_info<S, 64>();
    case 128: return play_info<S, 128>();
    case 256: return play_info<S, 256>();
    default: return play_info<S, 384>();
    }
}

template <class T> struct PTag { using type = T; };

template <class S, bool LES, int NXC>
struct PairBatchOps {
    using D = PairBatchDesc<S, LES, NXC>;
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
        PairMaps pm;
        void *const bufs[2] = {buf0, buf1};
        const char *cp = std::getenv("ISLBM_PAIR_COPIES");
        if (!(cp && std::strcmp(cp, "bulk") == 0) && make_pair_maps(k, (int)sizeof(S), bufs, &pm)) {
            std::memcpy((void *)d.tm, (const void *)pm.m, sizeof(d.tm));
            d.tm_on = 1;
        }
        std::memcpy(out, (const void *)&d, sizeof(d));
    }
    static cudaError_t prepare() {
        static bool attr_done = false;
        if (!attr_done) {
            cudaError_t e = cudaFuncSetAttribute(step_pair_batch_kernel<S, LES, NXC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)PLay<S, NXC>::smem_bytes);
            if (e != cudaSuccess) return e;
            attr_done = true;
        }
        return cudaSuccess;
    }
    static cudaError_t launch(const void *descs, const int2 *items, int nitems, int grid, int macros_on, cudaStream_t st) {
        cudaError_t e = prepare();
        if (e != cudaSuccess) return e;
        step_pair_batch_kernel<S, LES, NXC><<<grid, PLay<S, NXC>::NT, PLay<S, NXC>::smem_bytes, st>>>((const D *)descs, items,
                                                                                               nitems, macros_on);
        return cudaGetLastError();
    }
};

template <class F>
auto pdispatch(int precision, int NX, bool les, F &&f) {
    auto by_nx = [&](auto s_tag, auto les_tag) {
        using S = typename decltype(s_tag)::type;
        constexpr bool L = decltype(les_tag)::value;
        switch (NX) {
        case 32: return f(PairBatchOps<S, L, 32>{});
        case 64: return f(PairBatchOps<S, L, 64>{});
        case 128: return f(PairBatchOps<S, L, 128>{});
        case 256: return f(PairBatchOps<S, L, 256>{});
        default: return f(PairBatchOps<S, L, 384>{});
        }
    };
    auto by_les = [&](auto s_tag) { return les ? by_nx(s_tag, std::true_type{}) : by_nx(s_tag, std::false_type{}); };
    switch (precision) {
    case ISLBM_FP32: return by_les(PTag<float>{});
    case ISLBM_FP16_DEV: return by_les(PTag<__half>{});
    default: return by_les(PTag<__nv_bfloat16>{});
    }
}

}  // namespace

bool pair_supported(const StepConst &k, int precision) {
    if (precision == ISLBM_FP64) return false;
    if (k.NX != 32 && k.NX != 64 && k.NX != 128 && k.NX != 256 && k.NX != 384) return false;
    const int TY = k.NX <= 256 ? 256/k.NX : 1;
    return k.NY % TY == 0 && k.NY >= TY + 6 && k.NZ >= 8;
}

// Wall-normal segments per column for `tiles` tiles on `slots` resident CTAs: the count that
// minimises the estimated makespan (rounds of items x planes per item, a segment re-reading the
// 6 planes below it to fill its ring), each segment at least 16 targets long.
int pair_zsegs(int tiles, int slots, int NZ) {
    int best = 1;
    double best_cost = 1e300;
    for (int z = 1; z <= std::max(1, NZ/16); z++) {
        const int items = tiles*z;
        const int rounds = (items + slots - 1)/slots;
        const double cost = rounds*((double)NZ/z + 6.0);
        if (cost < best_cost - 1e-9) { best_cost = cost; best = z; }
    }
    return best;
}

int make_pair_const(const StepConst &k, int precision, const double *wx0, const double *wx2, const double *wy0,
                    const double *wy2, int num_sms, TiledConst *out) {
    TiledConst tc;
    std::memset(&tc, 0, sizeof(tc));
    const PLayInfo li = precision == ISLBM_FP32 ? play_for<float>(k.NX) : play_for<__half>(k.NX);
    tc.TY = li.ty;
    tc.smem_bytes = li.smem;
    for (int a = 0; a < 7; a++) {
        tc.wx[a] = make_float2((float)wx0[a], (float)wx2[a]);
        tc.wy[a] = make_float2((float)wy0[a], (float)wy2[a]);
        tc.wyb[0][a] = make_float2((float)wy0[a], (float)wy0[a]);
        tc.wyb[1][a] = make_float2((float)wy2[a], (float)wy2[a]);
    }
    // spanwise filter of aligned node pairs: node 0 (x0) sums w[k+3] v[x0+k] + w[k+4] v[x0+k+1]
    // over the pairs k = -4, -2, 0, 2; node 1 sums w[k+2] v[x0+k] + w[k+3] v[x0+k+1] over
    // k = -2, 0, 2, 4 (weights outside 0..6 are zero)
    for (int set = 0; set < 2; set++) {
        const double *w = set == 0 ? wx0 : wx2;
        auto W = [&](int i) { return (i >= 0 && i < 7) ? (float)w[i] : 0.f; };
        for (int kk = 0; kk < 4; kk++) {
            const int kx = -4 + 2*kk;
            tc.wxa[set][kk] = make_float2(W(kx + 3), W(kx + 4));
            const int ky = -2 + 2*kk;
            tc.wxb[set][kk] = make_float2(W(ky + 2), W(ky + 3));
        }
    }
    const int tiles = k.NY/tc.TY;
    const int per_sm = (int)std::min<size_t>((size_t)li.ctas_per_sm, (228*1024)/(tc.smem_bytes + 1024));
    const int slots = per_sm*num_sms;
    tc.zsegs = pair_zsegs(tiles, slots, k.NZ);
    if (const char *e = std::getenv("ISLBM_TILED_ZSEGS")) {   // tuning override
        const int z = std::atoi(e);
        if (z >= 1 && z <= k.NZ/8) tc.zsegs = z;
    }
    tc.grid = std::min(tiles*tc.zsegs, slots);
    *out = tc;
    return tc.smem_bytes <= 227*1024 ? 0 : -1;
}

bool make_pair_maps(const StepConst &k, int elem_bytes, void *const buf[2], PairMaps *out) {
    out->ok = false;
    if ((elem_bytes != 4 && elem_bytes != 2) || k.NX > 256 || !pair_supported(k, elem_bytes == 4 ? ISLBM_FP32 : ISLBM_FP16_DEV))
        return false;
    // the driver's encoder, looked up once (thread-safe static initialisation)
    static const PFN_cuTensorMapEncodeTiled_v12000 encode = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return nullptr;
        return (PFN_cuTensorMapEncodeTiled_v12000)fn;
    }();
    if (!encode) return false;
    const int TY = 256/k.NX;   // rows per tile of the paired layout (128 threads, two nodes each)
    const size_t es = (size_t)elem_bytes;
    const cuuint64_t dims[4] = {(cuuint64_t)k.NX, (cuuint64_t)k.NY, (cuuint64_t)k.NZ, 19};
    const cuuint64_t strides[3] = {k.NX*es, (size_t)k.NX*k.NY*es, (size_t)k.NX*k.NY*k.NZ*es};
    const cuuint32_t boxes[4][4] = {{(cuuint32_t)k.NX, (cuuint32_t)TY + 6, 1, 2}, {(cuuint32_t)k.NX, (cuuint32_t)TY + 6, 1, 4},
                                    {(cuuint32_t)k.NX, (cuuint32_t)TY, 1, 2}, {(cuuint32_t)k.NX, (cuuint32_t)TY, 1, 4}};
    const cuuint32_t unit[4] = {1, 1, 1, 1};
    const CUtensorMapDataType dt = elem_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_UINT16;
    for (int b = 0; b < 2; b++)
        for (int j = 0; j < 4; j++)
            if (encode(&out->m[b][j], dt, 4, buf[b], dims, strides, boxes[j], unit, CU_TENSOR_MAP_INTERLEAVE_NONE,
                       CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
                return false;
    out->buf[0] = buf[0];
    out->buf[1] = buf[1];
    out->ok = true;
    return true;
}

cudaError_t launch_step_pair(const StepLaunch &L) {
    switch (L.precision) {
    case ISLBM_FP32: return L.les ? launch_pnx<float, true>(L) : launch_pnx<float, false>(L);
    case ISLBM_FP16_DEV: return L.les ? launch_pnx<__half, true>(L) : launch_pnx<__half, false>(L);
    case ISLBM_BF16_DEV: return L.les ? launch_pnx<__nv_bfloat16, true>(L) : launch_pnx<__nv_bfloat16, false>(L);
    default: return cudaErrorNotSupported;
    }
}

size_t pair_batch_desc_bytes(int precision, int NX, bool les) {
    return pdispatch(precision, NX, les, [](auto ops) { return decltype(ops)::bytes(); });
}

void fill_pair_batch_desc(int precision, int NX, bool les, const Tables<float> &T, const StepConst &k, const TiledConst &tc,
                          Ctrl *ctrl, void *const macros[4], void *buf0, void *buf1, int ntiles, int nseg, void *out) {
    pdispatch(precision, NX, les, [&](auto ops) {
        decltype(ops)::fill(T, k, tc, ctrl, macros, buf0, buf1, ntiles, nseg, out);
        return 0;
    });
}

cudaError_t prepare_step_pair_batch(int precision, int NX, bool les) {
    return pdispatch(precision, NX, les, [&](auto ops) { return decltype(ops)::prepare(); });
}

cudaError_t launch_step_pair_batch(int precision, int NX, bool les, const void *descs, const int2 *items, int nitems,
                                   int grid, int macros_on, cudaStream_t stream) {
    return pdispatch(precision, NX, les,
                     [&](auto ops) { return decltype(ops)::launch(descs, items, nitems, grid, macros_on, stream); });
}

}  // namespace islbm
