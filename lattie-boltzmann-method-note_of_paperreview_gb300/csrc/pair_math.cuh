// Packed arithmetic on node pairs: every FP32 operation of the paired-node step kernel works
// on (node x, node x + 1) at once through the FP32x2 instructions of sm_100+ (add, mul and fma
// on a float2 in one instruction). A product followed by an addition or subtraction is
// contracted into one fused multiply-add, as the compiler does for scalar FP32 code.
#pragma once

#include <cuda_runtime.h>

#include "mrt_d3q19.cuh"

namespace islbm {

struct V2 {
    float2 v;
    __device__ __forceinline__ V2() {}
    __device__ __forceinline__ V2(float2 a) : v(a) {}
    __device__ __forceinline__ V2(float a, float b) : v(make_float2(a, b)) {}
    // broadcast constants (the generated MRT code writes T(c))
    __device__ __forceinline__ explicit V2(double c) : v(make_float2((float)c, (float)c)) {}
    __device__ __forceinline__ explicit V2(float c) : v(make_float2(c, c)) {}
    __device__ __forceinline__ explicit V2(int c) : v(make_float2((float)c, (float)c)) {}
};

__device__ __forceinline__ V2 vneg(V2 a) { return V2(-a.v.x, -a.v.y); }
__device__ __forceinline__ V2 vadd(V2 a, V2 b) { return V2(__fadd2_rn(a.v, b.v)); }
__device__ __forceinline__ V2 vsub(V2 a, V2 b) { return V2(__fadd2_rn(a.v, vneg(b).v)); }
__device__ __forceinline__ V2 vmul(V2 a, V2 b) { return V2(__fmul2_rn(a.v, b.v)); }
__device__ __forceinline__ V2 vfma(V2 a, V2 b, V2 c) { return V2(__ffma2_rn(a.v, b.v, c.v)); }

// a product not yet rounded: consumed by + or - as one fused multiply-add
struct V2M {
    V2 a, b;
    __device__ __forceinline__ operator V2() const { return vmul(a, b); }
};
__device__ __forceinline__ V2M operator*(V2 a, V2 b) { return V2M{a, b}; }
__device__ __forceinline__ V2M operator*(V2M m, V2 c) { return V2M{vmul(m.a, m.b), c}; }
__device__ __forceinline__ V2M operator*(V2 c, V2M m) { return V2M{c, vmul(m.a, m.b)}; }
__device__ __forceinline__ V2M operator*(V2M m, V2M n) { return V2M{vmul(m.a, m.b), vmul(n.a, n.b)}; }
__device__ __forceinline__ V2 operator+(V2 a, V2 b) { return vadd(a, b); }
__device__ __forceinline__ V2 operator-(V2 a, V2 b) { return vsub(a, b); }
__device__ __forceinline__ V2 operator-(V2 a) { return vneg(a); }
__device__ __forceinline__ V2 operator+(V2M m, V2 c) { return vfma(m.a, m.b, c); }
__device__ __forceinline__ V2 operator+(V2 c, V2M m) { return vfma(m.a, m.b, c); }
__device__ __forceinline__ V2 operator+(V2M m, V2M n) { return vfma(m.a, m.b, vmul(n.a, n.b)); }
__device__ __forceinline__ V2 operator-(V2 c, V2M m) { return vfma(vneg(m.a), m.b, c); }
__device__ __forceinline__ V2 operator-(V2M m, V2 c) { return vfma(m.a, m.b, vneg(c)); }
__device__ __forceinline__ V2 operator-(V2M m, V2M n) { return vfma(m.a, m.b, vneg(vmul(n.a, n.b))); }
__device__ __forceinline__ V2M operator-(V2M m) { return V2M{vneg(m.a), m.b}; }
__device__ __forceinline__ V2 &operator+=(V2 &a, V2 b) { a = vadd(a, b); return a; }
__device__ __forceinline__ V2 &operator-=(V2 &a, V2 b) { a = vsub(a, b); return a; }
__device__ __forceinline__ V2 &operator+=(V2 &a, V2M m) { a = vfma(m.a, m.b, a); return a; }
__device__ __forceinline__ V2 &operator-=(V2 &a, V2M m) { a = vfma(vneg(m.a), m.b, a); return a; }

// per-lane reciprocal and square root (no packed forms): the hardware approximations of the
// scalar FP32 collision
__device__ __forceinline__ V2 vrcp(V2 a) { return V2(__fdividef(1.f, a.v.x), __fdividef(1.f, a.v.y)); }
__device__ __forceinline__ float sqrt_nn(float v) { return v > 0.f ? v*rsqrtf(v) : 0.f; }

// Collision tail of C/evolution.h:597-652 for a node pair, the operator of collide_node_pairs
// (step_common.cuh) on packed pairs: mass correction, density and velocity from the opposite-
// direction pair sums and differences, their non-equilibrium parts, the Smagorinsky rate from
// Q = Pi:Pi (LES), the generated sparse MRT relaxation and the body force.
template <bool LES>
__device__ __forceinline__ void collide_x2(V2 (&F)[19], float rho_modify, float f6, float f12, float tau, float lesC,
                                           V2 &rho_s, V2 &u1, V2 &v1, V2 &w1) {
    constexpr int PA[9] = {1, 3, 5, 7, 8, 11, 12, 15, 16}, PB[9] = {2, 4, 6, 10, 9, 14, 13, 18, 17};
    F[0] = F[0] + V2(rho_modify);
    V2 S[9], A[9];
#pragma unroll
    for (int p = 0; p < 9; p++) { S[p] = F[PA[p]] + F[PB[p]]; A[p] = F[PA[p]] - F[PB[p]]; }
    const V2 r = ((F[0] + S[0]) + (S[1] + S[2])) + ((S[3] + S[4]) + (S[5] + S[6])) + (S[7] + S[8]);
    rho_s = r;
    const V2 inv = vrcp(r);
    u1 = vmul((A[0] + A[3]) + (A[5] - (A[4] + A[6])), inv);
    v1 = vmul((A[1] + A[3]) + (A[4] + (A[7] - A[8])), inv);
    w1 = vmul((A[2] + A[5]) + (A[6] + (A[7] + A[8])), inv);
    const V2 udot = u1*u1 + v1*v1 + w1*w1;
    const V2 base = V2(1.f) - V2(1.5f)*udot;
    // equilibrium of a pair: sum 2 w rho (base + 4.5 c^2), difference 6 w rho c (c = e_a . u)
    const V2 n2a1 = V2(-1.f/9.f)*r, n2a2 = V2(-1.f/18.f)*r;
    const V2 n6a1 = V2(-1.f/3.f)*r, n6a2 = V2(-1.f/6.f)*r;
    const V2 d0 = F[0] - (V2(1.f/3.f)*r)*base;
    {
        const V2 cu[9] = {u1, v1, w1, u1 + v1, v1 - u1, u1 + w1, w1 - u1, v1 + w1, w1 - v1};
#pragma unroll
        for (int p = 0; p < 9; p++) {
            const V2 t = (V2(4.5f)*cu[p])*cu[p] + base;
            S[p] = (p < 3 ? n2a1 : n2a2)*t + S[p];
            A[p] = (p < 3 ? n6a1 : n6a2)*cu[p] + A[p];
        }
    }
    V2 s_nu;
    if constexpr (LES) {
        const V2 Qn = pi_neq_norm2_pairs<V2>(S);
        const float nu0 = (tau - 0.5f)*(1.f/3.f);
        float sn[2];
#pragma unroll
        for (int l = 0; l < 2; l++) {
            const float q = l == 0 ? Qn.v.x : Qn.v.y;
            const float Sm = __fdividef(sqrt_nn(nu0*nu0 + 18.f*lesC*sqrt_nn(q)) - nu0, 6.f*lesC);
            sn[l] = __fdividef(1.f, tau + 3.f*lesC*Sm);
        }
        s_nu = V2(sn[0], sn[1]);
    } else {
        s_nu = V2(__fdividef(1.f, tau));
    }
    mrt_relax_pairs<V2>(F, d0, S, A, V2(1.19f), V2(1.4f), V2(1.2f), s_nu, V2(1.4f), V2(1.5f));
    const V2 p6 = V2(f6), p12 = V2(f12);
    F[3] += p6; F[4] -= p6;
    F[7] += p12; F[8] += p12; F[15] += p12; F[17] += p12;
    F[9] -= p12; F[10] -= p12; F[16] -= p12; F[18] -= p12;
}

}  // namespace islbm
