// Gather step kernel: one thread per unique node, every stencil value read through L1/L2.
//
// This is the direct form of stream_collide (C/evolution.h:358-684): the same departure-
// point interpolation in the same nesting order (x innermost, then y, then xi; F3/F4 with
// xi inside y as in C/interpolationHillISLBM.h:22-58), the wall bounce-back of :482-496, the
// BFL rows of :505-572 and the collision tail, with the periodic x/y wrap done by index
// arithmetic instead of ghost layers (periodicSW/periodicUD, :686-777). It serves any grid
// and every storage format, and is the parity path for FP64.
#include "step_common.cuh"
#include "step_launch.hpp"

namespace islbm {

namespace {

__device__ __forceinline__ int wrap(int v, int n) {
    v %= n;
    return v < 0 ? v + n : v;
}

template <class S, bool LES>
__global__ void __launch_bounds__(128) step_gather_kernel(const S *__restrict__ fo, S *__restrict__ fn,
                                                          Tables<typename Storage<S>::C> T, StepConst k,
                                                          Ctrl *ctrl, unsigned long long n, bool MACROS, bool MASS,
                                                          typename Storage<S>::C *rho_out,
                                                          typename Storage<S>::C *u_out,
                                                          typename Storage<S>::C *v_out,
                                                          typename Storage<S>::C *w_out) {
    using C = typename Storage<S>::C;
    const int NX = k.NX, NY = k.NY, NZ = k.NZ;
    const int x = blockIdx.x*blockDim.x + threadIdx.x;
    const int y = blockIdx.y*blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    const bool active = (x < NX) && (y < NY);
    const size_t N = (size_t)NX*NY*NZ;
    double ub = 0.0, mass = 0.0;
    const bool has_plane = (y == k.yplane);  // warp-uniform: a warp spans x at fixed y

    if (active) {
        int xs[7], ys[7];
#pragma unroll
        for (int a = 0; a < 7; a++) { xs[a] = wrap(x - 3 + a, NX); ys[a] = wrap(y - 3 + a, NY); }
        const int cz = min(max(z - 3, 0), NZ - 7);
        auto f = [&](int q, int xx, int yy, int zz) -> C {
            return load_f<S>(fo + (size_t)q*N, ((size_t)zz*NY + yy)*NX + xx, q);
        };
        const C *wxi = T.wxi + ((size_t)z*NY + y)*64;
        auto xiw = [&](int t, int c) -> C { return wxi[c*8 + t]; };
        auto wx = [&](const C *tab, int a) -> C { return tab[(size_t)a*NX + x]; };
        auto wy = [&](const C *tab, int b) -> C { return tab[(size_t)b*NY + y]; };

        C F[19];
        F[0] = f(0, x, y, z);
        // x-only (F1_Intrpl7, F2_Intrpl7)
        {
            C s1 = f(1, xs[0], y, z)*wx(T.wx0, 0), s2 = f(2, xs[0], y, z)*wx(T.wx2, 0);
#pragma unroll
            for (int a = 1; a < 7; a++) { s1 = s1 + f(1, xs[a], y, z)*wx(T.wx0, a); s2 = s2 + f(2, xs[a], y, z)*wx(T.wx2, a); }
            F[1] = s1; F[2] = s2;
        }
        // y (outer) x xi (inner) (F3_Intrpl7, F4_Intrpl7)
        {
            C o3 = 0, o4 = 0;
#pragma unroll
            for (int b = 0; b < 7; b++) {
                C i3 = f(3, x, ys[b], cz)*xiw(XI3, 0), i4 = f(4, x, ys[b], cz)*xiw(XI4, 0);
#pragma unroll
                for (int c = 1; c < 7; c++) { i3 = i3 + f(3, x, ys[b], cz + c)*xiw(XI3, c); i4 = i4 + f(4, x, ys[b], cz + c)*xiw(XI4, c); }
                o3 = b == 0 ? i3*wy(T.wy0, 0) : o3 + i3*wy(T.wy0, b);
                o4 = b == 0 ? i4*wy(T.wy2, 0) : o4 + i4*wy(T.wy2, b);
            }
            F[3] = o3; F[4] = o4;
        }
        // xi only (F5_Intrpl7, F6_Intrpl7)
        {
            C s5 = f(5, x, y, cz)*xiw(XI5, 0), s6 = f(6, x, y, cz)*xiw(XI6, 0);
#pragma unroll
            for (int c = 1; c < 7; c++) { s5 = s5 + f(5, x, y, cz + c)*xiw(XI5, c); s6 = s6 + f(6, x, y, cz + c)*xiw(XI6, c); }
            F[5] = s5; F[6] = s6;
        }
        // x, y, xi (X_Y_XI_Intrpl7) for F7..F10
        {
            const C *xt[4] = {T.wx0, T.wx2, T.wx0, T.wx2};
            const C *yt[4] = {T.wy0, T.wy0, T.wy2, T.wy2};
            const int zt[4] = {XI3, XI3, XI4, XI4};
#pragma unroll 1
            for (int m = 0; m < 4; m++) {
                const int q = 7 + m;
                C outer = 0;
#pragma unroll 1
                for (int c = 0; c < 7; c++) {
                    C mid = 0;
#pragma unroll
                    for (int b = 0; b < 7; b++) {
                        C in = f(q, xs[0], ys[b], cz + c)*wx(xt[m], 0);
#pragma unroll
                        for (int a = 1; a < 7; a++) in = in + f(q, xs[a], ys[b], cz + c)*wx(xt[m], a);
                        mid = b == 0 ? in*wy(yt[m], 0) : mid + in*wy(yt[m], b);
                    }
                    outer = c == 0 ? mid*xiw(zt[m], 0) : outer + mid*xiw(zt[m], c);
                }
                F[q] = outer;
            }
        }
        // x, xi (X_XI_Intrpl7) for F11..F14
        {
            const C *xt[4] = {T.wx0, T.wx2, T.wx0, T.wx2};
            const int zt[4] = {XI5, XI5, XI6, XI6};
#pragma unroll
            for (int m = 0; m < 4; m++) {
                const int q = 11 + m;
                C outer = 0;
#pragma unroll
                for (int c = 0; c < 7; c++) {
                    C in = f(q, xs[0], y, cz + c)*wx(xt[m], 0);
#pragma unroll
                    for (int a = 1; a < 7; a++) in = in + f(q, xs[a], y, cz + c)*wx(xt[m], a);
                    outer = c == 0 ? in*xiw(zt[m], 0) : outer + in*xiw(zt[m], c);
                }
                F[q] = outer;
            }
        }
        // y, xi (Y_XI_Intrpl7) for F15..F18
        {
            const C *yt[4] = {T.wy0, T.wy2, T.wy0, T.wy2};
            const int zt[4] = {XI15, XI16, XI17, XI18};
#pragma unroll
            for (int m = 0; m < 4; m++) {
                const int q = 15 + m;
                C outer = 0;
#pragma unroll
                for (int c = 0; c < 7; c++) {
                    C in = f(q, x, ys[0], cz + c)*wy(yt[m], 0);
#pragma unroll
                    for (int b = 1; b < 7; b++) in = in + f(q, x, ys[b], cz + c)*wy(yt[m], b);
                    outer = c == 0 ? in*xiw(zt[m], 0) : outer + in*xiw(zt[m], c);
                }
                F[q] = outer;
            }
        }
        // half-way bounce-back at the lower (k = 3) and upper (k = NZ6-4) walls
        if (z == 0) { F[5] = f(6, x, y, z); F[11] = f(14, x, y, z); F[12] = f(13, x, y, z); F[15] = f(18, x, y, z); F[16] = f(17, x, y, z); }
        if (z == NZ - 1) { F[6] = f(5, x, y, z); F[13] = f(12, x, y, z); F[14] = f(11, x, y, z); F[17] = f(16, x, y, z); F[18] = f(15, x, y, z); }
        // BFL on the first two rows above the hill
        if (z <= 1) {
            const int nb = 2*k.NYD6;
            const int r = z*k.NYD6 + (y + 3);
            const int ix = k.bfl_mode ? r : x + 3;   // reference: X weights at [i], Y weights at [j]
            const int iy = k.bfl_mode ? r : y + 3;
            auto bw = [&](int s, int a, int idx) -> C { return idx < nb ? T.bfl_w[((size_t)s*7 + a)*nb + idx] : C(0); };
            auto y_xi = [&](int q, int sy, int sz) -> C {   // Y_XI_Intrpl7 with k_c = 3
                C outer = 0;
#pragma unroll 1
                for (int c = 0; c < 7; c++) {
                    C in = f(q, x, ys[0], c)*bw(sy, 0, iy);
                    for (int b = 1; b < 7; b++) in = in + f(q, x, ys[b], c)*bw(sy, b, iy);
                    outer = c == 0 ? in*bw(sz, 0, r) : outer + in*bw(sz, c, r);
                }
                return outer;
            };
            auto xy_xi = [&](int q, int sx, int sy, int sz) -> C {   // X_Y_XI_Intrpl7 with k_c = 3
                C outer = 0;
#pragma unroll 1
                for (int c = 0; c < 7; c++) {
                    C mid = 0;
                    for (int b = 0; b < 7; b++) {
                        C in = f(q, xs[0], ys[b], c)*bw(sx, 0, ix);
                        for (int a = 1; a < 7; a++) in = in + f(q, xs[a], ys[b], c)*bw(sx, a, ix);
                        mid = b == 0 ? in*bw(sy, 0, iy) : mid + in*bw(sy, b, iy);
                    }
                    outer = c == 0 ? mid*bw(sz, 0, r) : outer + mid*bw(sz, c, r);
                }
                return outer;
            };
            auto lin = [&](C q, int a, int b) -> C {   // (1/(2Q)) f_a + ((2Q-1)/(2Q)) f_b at the node
                return (C(1)/(C(2)*q))*f(a, x, y, z) + ((C(2)*q - C(1))/(C(2)*q))*f(b, x, y, z);
            };
            if (T.bfl_flag[0*nb + r] == 1) {
                const C q = T.bfl_q[0*nb + r];
                if (q > C(0.5)) { F[3] = lin(q, 4, 3); F[7] = lin(q, 10, 7); F[8] = lin(q, 9, 8); }
                if (q < C(0.5)) {
                    F[3] = y_xi(4, B_YB378, B_XIB378);
                    F[7] = xy_xi(10, B_XB37, B_YB378, B_XIB378);
                    F[8] = xy_xi(9, B_XB38, B_YB378, B_XIB378);
                }
            }
            if (T.bfl_flag[1*nb + r] == 1) {
                const C q = T.bfl_q[1*nb + r];
                if (q > C(0.5)) { F[4] = lin(q, 3, 4); F[9] = lin(q, 8, 9); F[10] = lin(q, 7, 10); }
                if (q < C(0.5)) {
                    F[4] = y_xi(3, B_YB4910, B_XIB4910);
                    F[9] = xy_xi(8, B_XB49, B_YB4910, B_XIB4910);
                    F[10] = xy_xi(7, B_XB410, B_YB4910, B_XIB4910);
                }
            }
            if (T.bfl_flag[2*nb + r] == 1) {
                const C q = T.bfl_q[2*nb + r];
                if (q > C(0.5)) F[15] = lin(q, 18, 15);
                if (q < C(0.5)) F[15] = y_xi(18, B_YB15, B_XIB15);
            }
            if (T.bfl_flag[3*nb + r] == 1) {
                const C q = T.bfl_q[3*nb + r];
                if (q > C(0.5)) F[16] = lin(q, 17, 16);
                if (q < C(0.5)) F[16] = y_xi(17, B_YB16, B_XIB16);
            }
        }

        const double force = ctrl->force;
        const C f6 = (C)(1.0/6*force*k.dt), f12 = (C)(1.0/12*force*k.dt);
        C rho_s, u1, v1, w1;
        collide_node<C, LES>(F, (C)ctrl->rho_modify, f6, f12, (C)k.tau, (C)k.les_C, rho_s, u1, v1, w1);
        const size_t node = ((size_t)z*NY + y)*NX + x;
#pragma unroll
        for (int q = 0; q < 19; q++) store_f<S>(fn + (size_t)q*N, node, q, F[q]);
        if (MACROS) { rho_out[node] = rho_s; u_out[node] = u1; v_out[node] = v1; w_out[node] = w1; }
        if (has_plane) ub = (double)v1*T.dxv[x]*T.dzv[z];
        if (MASS) mass = (double)rho_s;
        if (!(rho_s == rho_s)) ctrl->nonfinite = 1u;
    }
    end_of_step<128>(ctrl, k, n, ub, mass, has_plane, MASS, gridDim.x*gridDim.y*gridDim.z);
}

template <class S, bool LES>
cudaError_t launch_t(const StepLaunch &L) {
    using C = typename Storage<S>::C;
    const dim3 block(32, 4, 1);
    const dim3 grid((L.k.NX + 31)/32, (L.k.NY + 3)/4, L.k.NZ);
    step_gather_kernel<S, LES><<<grid, block, 0, L.stream>>>(
        (const S *)L.fo, (S *)L.fn, *(const Tables<C> *)L.tables, L.k, L.ctrl, L.n, L.macros_on, L.mass,
        (C *)L.macros[0], (C *)L.macros[1], (C *)L.macros[2], (C *)L.macros[3]);
    return cudaGetLastError();
}

template <class S>
cudaError_t launch_s(const StepLaunch &L) {
    return L.les ? launch_t<S, true>(L) : launch_t<S, false>(L);
}

}  // namespace

cudaError_t launch_step_gather(const StepLaunch &L) {
    switch (L.precision) {
    case ISLBM_FP64: return launch_s<double>(L);
    case ISLBM_FP32: return launch_s<float>(L);
    case ISLBM_FP16_DEV: return launch_s<__half>(L);
    default: return launch_s<__nv_bfloat16>(L);
    }
}

}  // namespace islbm
