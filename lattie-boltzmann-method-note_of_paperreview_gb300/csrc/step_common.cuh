// Device-side pieces shared by every ISLBM step kernel: storage formats, table layout,
// the per-node collision tail and the end-of-step controller bookkeeping.
//
// Layout in HBM (one solve):
//   populations  19 arrays of N = NX*NY*NZ unique nodes, f[q][z][y][x] (x fastest),
//                two buffers (old/new) swapped every step; storage type S is double, float,
//                or half/bfloat16 holding the deviation f - ref_q (dev_ref below);
//   weights      per-x and per-y Lagrange weights [a][x], [a][y] and the xi weights of the
//                eight xi tables per (y, z), interleaved per stencil point a:
//                [(z*NY + y)*64 + a*8 + t] (t = F3,4,5,6,15,16,17,18);
//   BFL tables   flags, Q and the Q < 0.5 weights on the two wall rows, in the reference's
//                row indexing r = (k-3)*NYD6 + j (C/memory.h:125-145);
//   controller   body force, rho_modify, bulk-velocity accumulator (FP64, Ctrl below).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "mrt_d3q19.cuh"

namespace islbm {

template <class S> struct Storage;
template <> struct Storage<double> { using C = double; static constexpr bool dev = false; };
template <> struct Storage<float> { using C = float; static constexpr bool dev = false; };
template <> struct Storage<__half> { using C = float; static constexpr bool dev = true; };
template <> struct Storage<__nv_bfloat16> { using C = float; static constexpr bool dev = true; };

// D3Q19 lattice weights (C/initialization.h:10-12).
template <class C> __host__ __device__ __forceinline__ C lattice_w(int q) {
    return q == 0 ? C(1.0/3.0) : (q < 7 ? C(1.0/18.0) : C(1.0/36.0));
}

// Reference state of the deviation formats (FP16 / BF16 storage hold f_q - ref_q): the
// equilibrium at rho = 1 and the bulk flow u = (0, 0.05, 0) of the benchmark cases, so that
// the stored deviations are the small departures from the mean flow (about a third of the
// departures from rest). Any constant per direction gives the same step up to rounding, since
// every interpolation's weights sum to one and the reference is added back at each target.
__host__ __device__ __forceinline__ double dev_ref(int q) {
    const double u0 = 0.05;
    const int ey = (q == 3 || q == 7 || q == 8 || q == 15 || q == 17) ? 1
                 : (q == 4 || q == 9 || q == 10 || q == 16 || q == 18) ? -1 : 0;
    const double w = q == 0 ? 1.0/3.0 : (q < 7 ? 1.0/18.0 : 1.0/36.0);
    return w*(1.0 + 3.0*ey*u0 + 4.5*ey*ey*u0*u0 - 1.5*u0*u0);
}

__device__ __forceinline__ double to_c(double v) { return v; }
__device__ __forceinline__ float to_c(float v) { return v; }
__device__ __forceinline__ float to_c(__half v) { return __half2float(v); }
__device__ __forceinline__ float to_c(__nv_bfloat16 v) { return __bfloat162float(v); }

template <class S> __device__ __forceinline__ S from_c(typename Storage<S>::C v);
template <> __device__ __forceinline__ double from_c<double>(double v) { return v; }
template <> __device__ __forceinline__ float from_c<float>(float v) { return v; }
template <> __device__ __forceinline__ __half from_c<__half>(float v) { return __float2half_rn(v); }
template <> __device__ __forceinline__ __nv_bfloat16 from_c<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }

// full population value from storage (deviation formats add the reference state back)
template <class S> __device__ __forceinline__ typename Storage<S>::C load_f(const S *p, size_t i, int q) {
    using C = typename Storage<S>::C;
    const C v = to_c(__ldg(p + i));
    if constexpr (Storage<S>::dev) return v + (C)dev_ref(q); else return v;
}
template <class S> __device__ __forceinline__ void store_f(S *p, size_t i, int q, typename Storage<S>::C v) {
    using C = typename Storage<S>::C;
    if constexpr (Storage<S>::dev) p[i] = from_c<S>(v - (C)dev_ref(q)); else p[i] = from_c<S>(v);
}

// Controller state, FP64 (Force_d, rho_modify_d, Ub_avg_d of the reference, reduced to
// scalars; C/evolution.h:826-840, 1003-1042).
struct Ctrl {
    double force;            // body force along y
    double rho_modify;       // added to F0 in the next step
    double ub_acc;           // sum over the current controller window of the plane sums
    double ub_slot[2];       // plane sum of v*dx*dz of step n, slot n & 1
    double mass_slot[256];   // partial sums of rho on mass-check steps
    unsigned long long step; // completed steps
    unsigned int done;       // blocks finished in the running step
    unsigned int nonfinite;  // set when a non-finite density is produced
    unsigned int fault;      // set when a pipeline wait gave up (bounded waits)
};

template <class C> struct Tables {
    const C *wx0, *wx2;        // [a*NX + x], departure x -/+ minSize
    const C *wy0, *wy2;        // [a*NY + y], departure y -/+ minSize
    const C *wxi;              // [(z*NY + y)*64 + a*8 + t]
    const C *wxi2;             // the same as duplicated pairs, [(z*NY + y)*128 + a*16 + 2*t + {0, 1}]
                               // (FP32 tables only; the paired-node kernel's operand layout)
    const int *bfl_flag;       // [t*nb + r], t: F3, F4, F15, F16; nb = 2*NYD6
    const C *bfl_q;            // [t*nb + r]
    const C *bfl_w;            // [(s*7 + a)*nb + r], s: XB37 XB38 YB378 XiB378 XB49 XB410 YB4910 XiB4910 YB15 XiB15 YB16 XiB16
    const double *dxv;         // [x] (x[i+1]-x[i-1])/2 on the controller plane
    const double *dzv;         // [z] (z[k+1]-z[k-1])/2 on the controller plane
    const float *dxf, *dzf;    // the same in FP32 (per-column partial sums of the tiled kernel)
};

struct StepConst {
    int NX, NY, NZ, NYD6;
    int yplane;                // unique row of the reference's ghost row j = 0 (global row NY)
    int bfl_mode;
    int ndtfrc, mass_interval;
    double tau, les_C;         // relaxation time, Smagorinsky C = Cs^2 (0 = off)
    double dt;                 // = minSize
    double Uref, beta, area;   // controller: beta = max(0.001, 3/Re), area = LX*(LZ-1)
    double nnodes;
    int drill_plane;           // test hook: the tiled kernel never copies this plane (-1: off)
};

enum { XI3 = 0, XI4, XI5, XI6, XI15, XI16, XI17, XI18 };
enum { B_XB37 = 0, B_XB38, B_YB378, B_XIB378, B_XB49, B_XB410, B_YB4910, B_XIB4910, B_YB15, B_XIB15, B_YB16, B_XIB16 };

// Square root and reciprocal of the collision: IEEE in FP64 (the parity path); in FP32 the
// hardware approximations (a few ulp, no special-value branches), well inside the FP32
// tolerance of the step.
template <class C> __device__ __forceinline__ C my_sqrt(C v);
template <> __device__ __forceinline__ double my_sqrt<double>(double v) { return sqrt(v); }
template <> __device__ __forceinline__ float my_sqrt<float>(float v) { return v > 0.f ? v*rsqrtf(v) : 0.f; }
template <class C> __device__ __forceinline__ C my_rcp(C v);
template <> __device__ __forceinline__ double my_rcp<double>(double v) { return 1.0/v; }
template <> __device__ __forceinline__ float my_rcp<float>(float v) { return __fdividef(1.f, v); }
template <class C> __device__ __forceinline__ C my_div(C a, C b);
template <> __device__ __forceinline__ double my_div<double>(double a, double b) { return a/b; }
template <> __device__ __forceinline__ float my_div<float>(float a, float b) { return __fdividef(a, b); }

// Collision tail of C/evolution.h:597-652 for one node: mass correction, moments,
// equilibrium, MRT relaxation (optionally with the Smagorinsky rate) and body force.
// F holds the streamed populations on entry and the post-collision ones on exit.
template <class C, bool LES>
__device__ __forceinline__ void collide_node(C (&F)[19], C rho_modify, C f6, C f12, C tau, C lesC,
                                             C &rho_s, C &u1, C &v1, C &w1) {
    F[0] = F[0] + rho_modify;
    C r;
    if constexpr (sizeof(C) == 8) {
        // FP64: the reference's summation order (C/evolution.h:600-602)
        r = F[0];
#pragma unroll
        for (int q = 1; q < 19; q++) r = r + F[q];
    } else {
        // FP32: a balanced tree (depth 5 instead of a chain of 18 dependent adds)
        const C a0 = F[0] + F[1], a1 = F[2] + F[3], a2 = F[4] + F[5], a3 = F[6] + F[7], a4 = F[8] + F[9];
        const C a5 = F[10] + F[11], a6 = F[12] + F[13], a7 = F[14] + F[15], a8 = F[16] + F[17];
        r = (((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7))) + (a8 + F[18]);
    }
    rho_s = r;
    const C inv = my_rcp<C>(r);
    u1 = (F[1] + F[7] + F[9] + F[11] + F[13] - (F[2] + F[8] + F[10] + F[12] + F[14]))*inv;
    v1 = (F[3] + F[7] + F[8] + F[15] + F[17] - (F[4] + F[9] + F[10] + F[16] + F[18]))*inv;
    w1 = (F[5] + F[11] + F[12] + F[15] + F[16] - (F[6] + F[13] + F[14] + F[17] + F[18]))*inv;
    const C udot = u1*u1 + v1*v1 + w1*w1;
    const C a0 = C(1.0/3.0)*r, a1 = C(1.0/18.0)*r, a2 = C(1.0/36.0)*r;
    const C base = C(1) - C(1.5)*udot;
    C d[19];
    d[0] = F[0] - a0*base;
    {
        const C cu[9] = {u1, v1, w1, u1 + v1, -u1 + v1, u1 + w1, -u1 + w1, v1 + w1, -v1 + w1};
        const int qp[9] = {1, 3, 5, 7, 8, 11, 12, 15, 16};
        const int qm[9] = {2, 4, 6, 10, 9, 14, 13, 18, 17};
#pragma unroll
        for (int m = 0; m < 9; m++) {
            const C a = m < 3 ? a1 : a2;
            const C sym = base + C(4.5)*cu[m]*cu[m];
            const C asym = C(3)*cu[m];
            d[qp[m]] = F[qp[m]] - a*(sym + asym);
            d[qm[m]] = F[qm[m]] - a*(sym - asym);
        }
    }
    C s_nu = my_rcp<C>(tau);
    if constexpr (LES) {
        const C Qn = pi_neq_norm2(d);
        const C nu0 = (tau - C(0.5))*C(1.0/3.0);
        const C S = my_div<C>(my_sqrt<C>(nu0*nu0 + C(18)*lesC*my_sqrt<C>(Qn)) - nu0, C(6)*lesC);
        s_nu = my_rcp<C>(tau + C(3)*lesC*S);
    }
    mrt_relax<C>(F, d, C(1.19), C(1.4), C(1.2), s_nu, C(1.4), C(1.5));
    F[3] += f6; F[4] -= f6;
    F[7] += f12; F[8] += f12; F[15] += f12; F[17] += f12;
    F[9] -= f12; F[10] -= f12; F[16] -= f12; F[18] -= f12;
}

// FP32 collision of the tiled kernels: the operator of collide_node computed from the pair
// sums F[a] + F[b] and differences F[a] - F[b] of the opposite directions (a, b), so that
// density, momentum, the non-equilibrium pair sums/differences and the relaxation share them
// (the equilibrium part of a pair is 2 w rho (1 - 1.5 u.u + 4.5 c^2) in the sum and
// 6 w rho c in the difference, c = e_a . u).
template <bool LES>
__device__ __forceinline__ void collide_node_pairs(float (&F)[19], float rho_modify, float f6, float f12, float tau,
                                                   float lesC, float &rho_s, float &u1, float &v1, float &w1) {
    constexpr int PA[9] = {1, 3, 5, 7, 8, 11, 12, 15, 16}, PB[9] = {2, 4, 6, 10, 9, 14, 13, 18, 17};
    F[0] = F[0] + rho_modify;
    float S[9], A[9];
#pragma unroll
    for (int p = 0; p < 9; p++) { S[p] = F[PA[p]] + F[PB[p]]; A[p] = F[PA[p]] - F[PB[p]]; }
    const float r = ((F[0] + S[0]) + (S[1] + S[2])) + ((S[3] + S[4]) + (S[5] + S[6])) + (S[7] + S[8]);
    rho_s = r;
    const float inv = my_rcp<float>(r);
    u1 = ((A[0] + A[3]) + (A[5] - (A[4] + A[6])))*inv;
    v1 = ((A[1] + A[3]) + (A[4] + (A[7] - A[8])))*inv;
    w1 = ((A[2] + A[5]) + (A[6] + (A[7] + A[8])))*inv;
    const float udot = u1*u1 + v1*v1 + w1*w1;
    const float base = 1.f - 1.5f*udot;
    const float a1 = (1.f/18.f)*r, a2 = (1.f/36.f)*r;
    const float d0 = F[0] - (1.f/3.f)*r*base;
    {
        const float cu[9] = {u1, v1, w1, u1 + v1, -u1 + v1, u1 + w1, -u1 + w1, v1 + w1, -v1 + w1};
#pragma unroll
        for (int p = 0; p < 9; p++) {
            const float a = p < 3 ? a1 : a2;
            S[p] = S[p] - 2.f*a*(base + 4.5f*cu[p]*cu[p]);
            A[p] = A[p] - 6.f*a*cu[p];
        }
    }
    float s_nu = my_rcp<float>(tau);
    if constexpr (LES) {
        const float Qn = pi_neq_norm2_pairs(S);
        const float nu0 = (tau - 0.5f)*(1.f/3.f);
        const float Sm = my_div<float>(my_sqrt<float>(nu0*nu0 + 18.f*lesC*my_sqrt<float>(Qn)) - nu0, 6.f*lesC);
        s_nu = my_rcp<float>(tau + 3.f*lesC*Sm);
    }
    mrt_relax_pairs<float>(F, d0, S, A, 1.19f, 1.4f, 1.2f, s_nu, 1.4f, 1.5f);
    F[3] += f6; F[4] -= f6;
    F[7] += f12; F[8] += f12; F[15] += f12; F[17] += f12;
    F[9] -= f12; F[10] -= f12; F[16] -= f12; F[18] -= f12;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// End-of-step bookkeeping, run by the last block of the step kernel (after every block has
// added its partial sums): bulk-velocity window, forcing controller every NDTFRC steps
// (C/evolution.h:1003-1042) and the mass correction for the next step.
__device__ __forceinline__ void finish_step(Ctrl *ctrl, const StepConst &k, unsigned long long n, bool mass_step) {
    // other blocks updated these with atomics during this kernel: read them from L2
    double acc = __ldcg(&ctrl->ub_acc) + __ldcg(&ctrl->ub_slot[(n - 1) & 1]);
    ctrl->ub_slot[(n - 1) & 1] = 0.0;
    double force = __ldcg(&ctrl->force);
    if (n % (unsigned long long)k.ndtfrc == 0ULL) {
        const double ub = acc/k.area/(double)k.ndtfrc;
        force = force + k.beta*(k.Uref - ub)*k.Uref/3.036;
        acc = 0.0;
    }
    ctrl->ub_acc = acc;
    ctrl->force = force;
    if (mass_step) {
        double m = 0.0;
        for (int i = 0; i < 256; i++) { m += __ldcg(&ctrl->mass_slot[i]); ctrl->mass_slot[i] = 0.0; }
        ctrl->rho_modify = (k.nnodes - m)/k.nnodes;
        if (!(m == m)) ctrl->nonfinite = 1u;
    } else {
        ctrl->rho_modify = 0.0;
    }
    ctrl->step = n;
    ctrl->done = 0u;
}

// Block-level end of step: reduce the plane and mass partials and let the last block run
// finish_step. `ub` and `mass` are this thread's contributions (0 when not applicable).
// `n` is the 1-based number of the step being computed. `has_plane` must be uniform
// within a warp (every kernel maps a warp to nodes of one y row).
// `total` is the number of blocks (or work items) that report to this controller per step.
template <int NTHREADS>
__device__ __forceinline__ void end_of_step(Ctrl *ctrl, const StepConst &k, unsigned long long n, double ub,
                                            double mass, bool has_plane, bool mass_step, unsigned total) {
    __shared__ double red[2][NTHREADS/32];
    __shared__ int any_plane;
    __shared__ bool last;
    const int tid = threadIdx.x + blockDim.x*(threadIdx.y + blockDim.y*threadIdx.z);
    const int lane = tid & 31, warp = tid >> 5;
    const unsigned bid = blockIdx.x + gridDim.x*(blockIdx.y + gridDim.y*blockIdx.z);
    if (tid == 0) any_plane = 0;
    __syncthreads();
    ub = has_plane ? warp_sum(ub) : 0.0;
    if (lane == 0) {
        red[0][warp] = ub;
        if (has_plane) any_plane = 1;
    }
    if (mass_step) {
        mass = warp_sum(mass);
        if (lane == 0) red[1][warp] = mass;
    }
    __syncthreads();
    if (tid == 0) {
        if (any_plane) {
            double s = 0.0;
            for (int w = 0; w < NTHREADS/32; w++) s += red[0][w];
            atomicAdd(&ctrl->ub_slot[n & 1ULL], s);
        }
        if (mass_step) {
            double s = 0.0;
            for (int w = 0; w < NTHREADS/32; w++) s += red[1][w];
            atomicAdd(&ctrl->mass_slot[bid & 255u], s);
        }
        __threadfence();
        last = (atomicAdd(&ctrl->done, 1u) == total - 1u);
    }
    __syncthreads();
    if (last && tid == 0) {
        __threadfence();
        finish_step(ctrl, k, n, mass_step);
    }
}

}  // namespace islbm
