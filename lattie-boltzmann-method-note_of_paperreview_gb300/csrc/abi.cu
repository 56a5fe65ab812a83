// C ABI of the ISLBM step library (declared in include/islbm.h).
//
// islbm_init does the reference's one-time setup on the host in FP64 (geometry.cpp), packs
// the tables for the unique-node device layout, uploads them with the initial state; the
// step loop then runs one fused kernel per lattice step on the handle's stream. All device
// memory is owned by the handle; errors come back as islbm_status codes.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/islbm.h"
#include "../../include/islbm_testing.h"
#include "geometry.hpp"
#include "step_launch.hpp"
#include "step_tiled.hpp"
#include "handle.hpp"

using namespace islbm;

namespace {

thread_local std::string g_last;

template <class T> struct Tag { using type = T; };

int cuda_fail(cudaError_t e, const char *what) {
    g_last = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return ISLBM_ERR_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return ISLBM_ERR_NO_DEVICE;
    return ISLBM_ERR_CUDA;
}

#define CK(call)                                                  \
    do {                                                          \
        cudaError_t e_ = (call);                                  \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);       \
    } while (0)

size_t storage_bytes(int precision) {
    switch (precision) {
    case ISLBM_FP64: return 8;
    case ISLBM_FP32: return 4;
    default: return 2;
    }
}
size_t compute_bytes(int precision) { return precision == ISLBM_FP64 ? 8 : 4; }

// table sizes in compute-type elements
struct TabSizes {
    size_t wx, wy, wxi, wxi2, bq, bw, flags_bytes, dxv, dzv;
};
TabSizes tab_sizes(const islbm_params &p) {
    TabSizes s{};
    const size_t nb = 2*(size_t)(p.NY + 7);
    s.wx = 7*(size_t)p.NX; s.wy = 7*(size_t)p.NY;
    s.wxi = (size_t)p.NZ*p.NY*64;
    s.wxi2 = p.precision == ISLBM_FP64 ? 0 : (size_t)p.NZ*p.NY*128;
    s.bq = 4*nb; s.bw = (size_t)Geometry::NBFL*7*nb;
    s.flags_bytes = 4*nb*sizeof(int);
    s.dxv = (size_t)p.NX; s.dzv = (size_t)p.NZ;
    return s;
}
size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }
size_t tables_bytes(const islbm_params &p) {
    const TabSizes s = tab_sizes(p);
    const size_t c = compute_bytes(p.precision);
    return align256(2*s.wx*c) + align256(2*s.wy*c) + align256(s.wxi*c) + align256(s.wxi2*c) + align256(s.bq*c) + align256(s.bw*c) +
           align256(s.flags_bytes) + align256(s.dxv*8) + align256(s.dzv*8) + align256(s.dxv*4) + align256(s.dzv*4);
}

size_t required_bytes(const islbm_params &p) {
    const size_t N = (size_t)p.NX*p.NY*p.NZ;
    return 2*19*N*storage_bytes(p.precision) + 4*N*compute_bytes(p.precision) + tables_bytes(p) + align256(sizeof(Ctrl));
}

// unique node (x, y, z) <-> reference index (i, j, k)
inline size_t uidx(const islbm_handle *h, int x, int y, int z) { return ((size_t)z*h->p.NY + y)*h->p.NX + x; }

template <class C>
void pack_tables(const Geometry &g, const islbm_params &p, std::vector<char> &blob, Tables<C> &t, char *dev_base) {
    const TabSizes s = tab_sizes(p);
    const int NX = p.NX, NY = p.NY, NZ = p.NZ, NX6 = g.NX6, NYD6 = g.NYD6, NZ6 = g.NZ6;
    const size_t nb = 2*(size_t)NYD6, nyz = (size_t)NYD6*NZ6;
    blob.assign(tables_bytes(p), 0);
    size_t off = 0;
    auto take = [&](size_t bytes) { char *hp = blob.data() + off; char *dp = dev_base + off; off += align256(bytes); return std::make_pair(hp, dp); };
    auto [hx, dx] = take(2*s.wx*sizeof(C));
    C *wx = (C *)hx;
    for (int a = 0; a < 7; a++)
        for (int x = 0; x < NX; x++) {
            wx[(size_t)a*NX + x] = (C)g.XP0[(size_t)a*NX6 + x + 3];
            wx[s.wx + (size_t)a*NX + x] = (C)g.XP2[(size_t)a*NX6 + x + 3];
        }
    t.wx0 = (const C *)dx; t.wx2 = (const C *)dx + s.wx;
    auto [hy, dy] = take(2*s.wy*sizeof(C));
    C *wy = (C *)hy;
    for (int a = 0; a < 7; a++)
        for (int y = 0; y < NY; y++) {
            wy[(size_t)a*NY + y] = (C)g.YP0[(size_t)a*NYD6 + y + 3];
            wy[s.wy + (size_t)a*NY + y] = (C)g.YP2[(size_t)a*NYD6 + y + 3];
        }
    t.wy0 = (const C *)dy; t.wy2 = (const C *)dy + s.wy;
    auto [hxi, dxi] = take(s.wxi*sizeof(C));
    C *wxi = (C *)hxi;
    for (int z = 0; z < NZ; z++)
        for (int y = 0; y < NY; y++)
            for (int tt = 0; tt < 8; tt++)
                for (int a = 0; a < 7; a++)
                    wxi[((size_t)z*NY + y)*64 + a*8 + tt] = (C)g.XiT[((size_t)tt*7 + a)*nyz + (size_t)(y + 3)*NZ6 + (z + 3)];
    t.wxi = (const C *)dxi;
    auto [hxi2, dxi2] = take(s.wxi2*sizeof(C));
    C *wxi2 = (C *)hxi2;
    for (size_t r = 0; r < s.wxi2/128; r++)
        for (int a = 0; a < 8; a++)
            for (int tt = 0; tt < 8; tt++) {
                const C v = a < 7 ? wxi[r*64 + a*8 + tt] : (C)0;
                wxi2[r*128 + a*16 + 2*tt] = v;
                wxi2[r*128 + a*16 + 2*tt + 1] = v;
            }
    t.wxi2 = s.wxi2 ? (const C *)dxi2 : nullptr;
    auto [hq, dq] = take(s.bq*sizeof(C));
    for (size_t i = 0; i < s.bq; i++) ((C *)hq)[i] = (C)g.Q[i];
    t.bfl_q = (const C *)dq;
    auto [hw, dw] = take(s.bw*sizeof(C));
    for (size_t i = 0; i < s.bw; i++) ((C *)hw)[i] = (C)g.BW[i];
    t.bfl_w = (const C *)dw;
    auto [hf, df] = take(s.flags_bytes);
    std::memcpy(hf, g.bfl.data(), s.flags_bytes);
    t.bfl_flag = (const int *)df;
    // controller plane: the reference's ghost row j = 0 (AccumulateUbulk, C/evolution.h:836-837)
    auto [hdx, ddx] = take(s.dxv*8);
    for (int x = 0; x < NX; x++) ((double *)hdx)[x] = (g.x[x + 4] - g.x[x + 2])/2.0;
    t.dxv = (const double *)ddx;
    auto [hdz, ddz] = take(s.dzv*8);
    for (int z = 0; z < NZ; z++) ((double *)hdz)[z] = (g.z[(size_t)0*NZ6 + z + 4] - g.z[(size_t)0*NZ6 + z + 2])/2.0;
    t.dzv = (const double *)ddz;
    auto [hdxf, ddxf] = take(s.dxv*4);
    for (int x = 0; x < NX; x++) ((float *)hdxf)[x] = (float)((double *)hdx)[x];
    t.dxf = (const float *)ddxf;
    auto [hdzf, ddzf] = take(s.dzv*4);
    for (int z = 0; z < NZ; z++) ((float *)hdzf)[z] = (float)((double *)hdz)[z];
    t.dzf = (const float *)ddzf;
    (void)nb;
}

// equilibrium of the initial state (InitialUsingDftFunc, C/initialization.h:36-42)
void initial_node(const islbm_handle *h, int x, int y, int z, double *rho, double *u, double *v, double *w, double f[19]) {
    static const int E[19][3] = {{0,0,0},{1,0,0},{-1,0,0},{0,1,0},{0,-1,0},{0,0,1},{0,0,-1},{1,1,0},{-1,1,0},{1,-1,0},
                                 {-1,-1,0},{1,0,1},{-1,0,1},{1,0,-1},{-1,0,-1},{0,1,1},{0,-1,1},{0,1,-1},{0,-1,-1}};
    static const double W[19] = {(1.0/3.0),(1.0/18.0),(1.0/18.0),(1.0/18.0),(1.0/18.0),(1.0/18.0),(1.0/18.0),
                                 (1.0/36.0),(1.0/36.0),(1.0/36.0),(1.0/36.0),(1.0/36.0),(1.0/36.0),(1.0/36.0),
                                 (1.0/36.0),(1.0/36.0),(1.0/36.0),(1.0/36.0),(1.0/36.0)};
    double rr = 1.0, uu = 0.0, vv = 0.0, ww = 0.0;
    if (h->p.init_mode == 1) {
        // counter-based noise: splitmix64(seed + golden*(3*node + comp + 1)) -> [-1, 1)
        const unsigned long long node = ((unsigned long long)z*h->p.NY + y)*h->p.NX + x;
        double r3[3];
        for (int c = 0; c < 3; c++) {
            unsigned long long s = h->p.seed + 0x9E3779B97F4A7C15ULL*(3ULL*node + (unsigned long long)c + 1ULL);
            s = (s ^ (s >> 30))*0xBF58476D1CE4E5B9ULL;
            s = (s ^ (s >> 27))*0x94D049BB133111EBULL;
            s = s ^ (s >> 31);
            r3[c] = (double)(s >> 11)*(1.0/9007199254740992.0)*2.0 - 1.0;
        }
        const double ub = h->p.Uref, amp = h->p.perturb;
        uu = ub*amp*r3[0];
        vv = ub + ub*amp*r3[1];
        ww = ub*amp*r3[2];
    }
    *rho = rr; *u = uu; *v = vv; *w = ww;
    const double udot = uu*uu + vv*vv + ww*ww;
    f[0] = W[0]*rr*(1.0 - 1.5*udot);
    for (int q = 1; q < 19; q++) {
        const double eu = (double)E[q][0]*uu + (double)E[q][1]*vv + (double)E[q][2]*ww;
        f[q] = W[q]*rr*(1.0 + 3.0*eu + 4.5*eu*eu - 1.5*udot);
    }
}

// Device form of initial_node for every unique node: the same FP64 operations in the same
// order, each rounded on its own (no contraction), so the state equals the host computation
// bit for bit; then stored in the storage format as to_storage does.
__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }
template <class S> __device__ __forceinline__ S to_s(double f, double wq);
template <> __device__ __forceinline__ double to_s<double>(double f, double) { return f; }
template <> __device__ __forceinline__ float to_s<float>(double f, double) { return __double2float_rn(f); }
template <> __device__ __forceinline__ __half to_s<__half>(double f, double wq) { return __float2half_rn(__double2float_rn(ds(f, wq))); }
template <> __device__ __forceinline__ __nv_bfloat16 to_s<__nv_bfloat16>(double f, double wq) {
    return __float2bfloat16_rn(__double2float_rn(ds(f, wq)));
}

template <class S, class C>
__global__ void init_state_kernel(S *f, C *rho, C *u, C *v, C *w, size_t N, unsigned long long seed, int mode, double ub,
                                  double amp) {
    const double W[3] = {1.0/3.0, 1.0/18.0, 1.0/36.0};
    const signed char E[19][3] = {{0,0,0},{1,0,0},{-1,0,0},{0,1,0},{0,-1,0},{0,0,1},{0,0,-1},{1,1,0},{-1,1,0},{1,-1,0},
                                  {-1,-1,0},{1,0,1},{-1,0,1},{1,0,-1},{-1,0,-1},{0,1,1},{0,-1,1},{0,1,-1},{0,-1,-1}};
    for (size_t i = blockIdx.x*(size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x*blockDim.x) {
        double rr = 1.0, uu = 0.0, vv = 0.0, ww = 0.0;
        if (mode == 1) {
            double r3[3];
            for (int c = 0; c < 3; c++) {
                unsigned long long s = seed + 0x9E3779B97F4A7C15ULL*(3ULL*i + (unsigned long long)c + 1ULL);
                s = (s ^ (s >> 30))*0xBF58476D1CE4E5B9ULL;
                s = (s ^ (s >> 27))*0x94D049BB133111EBULL;
                s = s ^ (s >> 31);
                r3[c] = ds(dm(dm((double)(s >> 11), 1.0/9007199254740992.0), 2.0), 1.0);
            }
            const double ua = dm(ub, amp);
            uu = dm(ua, r3[0]);
            vv = da(ub, dm(ua, r3[1]));
            ww = dm(ua, r3[2]);
        }
        rho[i] = (C)rr; u[i] = (C)uu; v[i] = (C)vv; w[i] = (C)ww;
        const double udot = da(da(dm(uu, uu), dm(vv, vv)), dm(ww, ww));
        f[i] = to_s<S>(dm(dm(W[0], rr), ds(1.0, dm(1.5, udot))), dev_ref(0));
        for (int q = 1; q < 19; q++) {
            const double eu = da(da(dm((double)E[q][0], uu), dm((double)E[q][1], vv)), dm((double)E[q][2], ww));
            const double wq = W[q < 7 ? 1 : 2];
            const double fq = dm(dm(wq, rr), ds(da(da(1.0, dm(3.0, eu)), dm(dm(4.5, eu), eu)), dm(1.5, udot)));
            f[(size_t)q*N + i] = to_s<S>(fq, dev_ref(q));
        }
    }
}

cudaError_t launch_init_state(const islbm_handle *h, void *f) {
    const unsigned grid = (unsigned)std::min<size_t>(4096, (h->N + 255)/256);
    const auto &p = h->p;
    auto go = [&](auto s_tag, auto c_tag) {
        using S = typename decltype(s_tag)::type;
        using C = typename decltype(c_tag)::type;
        init_state_kernel<S, C><<<grid, 256, 0, h->stream>>>((S *)f, (C *)h->macros[0], (C *)h->macros[1],
                                                              (C *)h->macros[2], (C *)h->macros[3], h->N, p.seed,
                                                              p.init_mode, p.Uref, p.perturb);
        return cudaGetLastError();
    };
    switch (p.precision) {
    case ISLBM_FP64: return go(Tag<double>{}, Tag<double>{});
    case ISLBM_FP32: return go(Tag<float>{}, Tag<float>{});
    case ISLBM_FP16_DEV: return go(Tag<__half>{}, Tag<float>{});
    default: return go(Tag<__nv_bfloat16>{}, Tag<float>{});
    }
}

// Device forms of to_storage / from_storage (same operations, same rounding) for the unique
// layout, so that host buffers move as FP64 without host-side conversion loops.
template <class S>
__global__ void to_storage_kernel(const double *__restrict__ src, S *__restrict__ dst, size_t n, double wq) {
    for (size_t i = blockIdx.x*(size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x*blockDim.x)
        dst[i] = to_s<S>(src[i], wq);
}
template <class S> __device__ __forceinline__ double from_s(S v, float wq);
template <> __device__ __forceinline__ double from_s<double>(double v, float) { return v; }
template <> __device__ __forceinline__ double from_s<float>(float v, float) { return (double)v; }
template <> __device__ __forceinline__ double from_s<__half>(__half v, float wq) { return (double)__fadd_rn(__half2float(v), wq); }
template <> __device__ __forceinline__ double from_s<__nv_bfloat16>(__nv_bfloat16 v, float wq) {
    return (double)__fadd_rn(__bfloat162float(v), wq);
}
template <class S>
__global__ void from_storage_kernel(const S *__restrict__ src, double *__restrict__ dst, size_t n, float wq) {
    for (size_t i = blockIdx.x*(size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x*blockDim.x)
        dst[i] = from_s<S>(src[i], wq);
}

template <class F>
cudaError_t by_storage(int precision, F &&f) {
    switch (precision) {
    case ISLBM_FP64: return f(Tag<double>{});
    case ISLBM_FP32: return f(Tag<float>{});
    case ISLBM_FP16_DEV: return f(Tag<__half>{});
    default: return f(Tag<__nv_bfloat16>{});
    }
}

// the FP64 transfer buffer of a handle (N doubles, allocated on first use)
cudaError_t xfer_buffer(islbm_handle *h) {
    if (h->xfer) return cudaSuccess;
    return cudaMalloc(&h->xfer, h->N*sizeof(double));
}

unsigned conv_grid(size_t n) { return (unsigned)std::min<size_t>(4096, (n + 255)/256); }

// host <-> storage conversion of one population array
void to_storage(int precision, int q, const double *src, void *dst, size_t n) {
    const double wq = dev_ref(q);
    switch (precision) {
    case ISLBM_FP64: std::memcpy(dst, src, n*8); break;
    case ISLBM_FP32: for (size_t i = 0; i < n; i++) ((float *)dst)[i] = (float)src[i]; break;
    case ISLBM_FP16_DEV: for (size_t i = 0; i < n; i++) ((__half *)dst)[i] = __float2half_rn((float)(src[i] - wq)); break;
    default: for (size_t i = 0; i < n; i++) ((__nv_bfloat16 *)dst)[i] = __float2bfloat16_rn((float)(src[i] - wq)); break;
    }
}
void from_storage(int precision, int q, const void *src, double *dst, size_t n) {
    const float wq = (float)dev_ref(q);
    switch (precision) {
    case ISLBM_FP64: std::memcpy(dst, src, n*8); break;
    case ISLBM_FP32: for (size_t i = 0; i < n; i++) dst[i] = ((const float *)src)[i]; break;
    case ISLBM_FP16_DEV: for (size_t i = 0; i < n; i++) dst[i] = (double)(__half2float(((const __half *)src)[i]) + wq); break;
    default: for (size_t i = 0; i < n; i++) dst[i] = (double)(__bfloat162float(((const __nv_bfloat16 *)src)[i]) + wq); break;
    }
}

// unique [z][y][x] -> reference layout (NYD6, NZ6, NX6) with periodic ghosts and duplicates
void unique_to_reference(const islbm_handle *h, const double *u, double *r) {
    const int NX = h->p.NX, NY = h->p.NY, NZ = h->p.NZ, NX6 = NX + 7, NYD6 = NY + 7, NZ6 = NZ + 6;
    std::memset(r, 0, (size_t)NX6*NYD6*NZ6*sizeof(double));
    for (int j = 0; j < NYD6; j++) {
        const int y = ((j - 3) % NY + NY) % NY;
        for (int k = 3; k < NZ6 - 3; k++)
            for (int i = 0; i < NX6; i++) {
                const int x = ((i - 3) % NX + NX) % NX;
                r[(size_t)j*NX6*NZ6 + (size_t)k*NX6 + i] = u[uidx(h, x, y, k - 3)];
            }
    }
}
void reference_to_unique(const islbm_handle *h, const double *r, double *u) {
    const int NX = h->p.NX, NY = h->p.NY, NZ = h->p.NZ, NX6 = NX + 7, NZ6 = NZ + 6;
    for (int z = 0; z < NZ; z++)
        for (int y = 0; y < NY; y++)
            for (int x = 0; x < NX; x++)
                u[uidx(h, x, y, z)] = r[(size_t)(y + 3)*NX6*NZ6 + (size_t)(z + 3)*NX6 + (x + 3)];
}

int check_handle(const islbm_handle *h) { return h ? ISLBM_OK : ISLBM_ERR_INVALID_ARGUMENT; }

int copy_macro(islbm_handle *h, int which, double *out, int layout) {
    const size_t N = h->N;
    if (layout == ISLBM_LAYOUT_UNIQUE && h->celem == 4) {
        // widen on the device and copy straight into the caller's buffer
        CK(xfer_buffer(h));
        from_storage_kernel<float><<<conv_grid(N), 256, 0, h->stream>>>((const float *)h->macros[which], h->xfer, N, 0.f);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(out, h->xfer, N*8, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        return ISLBM_OK;
    }
    std::vector<double> tmp(N);
    if (h->celem == 8) {
        CK(cudaMemcpyAsync(tmp.data(), h->macros[which], N*8, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
    } else {
        std::vector<float> f(N);
        CK(cudaMemcpyAsync(f.data(), h->macros[which], N*4, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        for (size_t i = 0; i < N; i++) tmp[i] = f[i];
    }
    if (layout == ISLBM_LAYOUT_REFERENCE) unique_to_reference(h, tmp.data(), out);
    else std::memcpy(out, tmp.data(), N*8);
    return ISLBM_OK;
}

void free_handle_impl(islbm_handle *h) {
    if (!h) return;
    cudaSetDevice(h->device);
    for (int b = 0; b < 2; b++) if (h->fbuf[b]) cudaFree(h->fbuf[b]);
    for (int m = 0; m < 4; m++) if (h->macros[m]) cudaFree(h->macros[m]);
    if (h->tabmem) cudaFree(h->tabmem);
    if (h->ctrl) cudaFree(h->ctrl);
    if (h->stats) cudaFree(h->stats);
    if (h->zslope) cudaFree(h->zslope);
    if (h->xfer) cudaFree(h->xfer);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

int init_impl(const islbm_params *pp, islbm_handle *h) {
    h->p = *pp;
    const int st = h->g.build(*pp);
    if (st != ISLBM_OK) { g_last = "invalid parameters"; return st; }
    const islbm_params &p = h->p;
    if (p.hbm_budget_bytes && required_bytes(p) > p.hbm_budget_bytes) { g_last = "HBM budget exceeded"; return ISLBM_ERR_HBM_BUDGET; }
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) { g_last = "no CUDA device"; return ISLBM_ERR_NO_DEVICE; }
    if (p.device < 0 || p.device >= ndev) return ISLBM_ERR_INVALID_ARGUMENT;
    h->device = p.device;
    CK(cudaSetDevice(h->device));
    CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    h->N = (size_t)p.NX*p.NY*p.NZ;
    h->elem = storage_bytes(p.precision);
    h->celem = compute_bytes(p.precision);
    for (int b = 0; b < 2; b++) CK(cudaMalloc(&h->fbuf[b], 19*h->N*h->elem));
    for (int m = 0; m < 4; m++) CK(cudaMalloc(&h->macros[m], h->N*h->celem));
    h->tab_bytes = tables_bytes(p);
    CK(cudaMalloc(&h->tabmem, h->tab_bytes));
    CK(cudaMalloc(&h->ctrl, sizeof(Ctrl)));

    std::vector<char> blob;
    if (p.precision == ISLBM_FP64) pack_tables<double>(h->g, p, blob, h->td, (char *)h->tabmem);
    else pack_tables<float>(h->g, p, blob, h->tf, (char *)h->tabmem);
    CK(cudaMemcpyAsync(h->tabmem, blob.data(), blob.size(), cudaMemcpyHostToDevice, h->stream));

    // initial state on the unique nodes, computed on the device
    CK(launch_init_state(h, h->fbuf[0]));

    // step constants and controller
    StepConst &k = h->k;
    k.NX = p.NX; k.NY = p.NY; k.NZ = p.NZ; k.NYD6 = h->g.NYD6;
    k.yplane = ((0 - 3) % p.NY + p.NY) % p.NY;   // reference ghost row j = 0 holds global row NY
    k.bfl_mode = p.bfl_mode;
    k.ndtfrc = p.NDTFRC; k.mass_interval = p.mass_interval;
    k.tau = h->g.tau; k.les_C = p.les_cs*p.les_cs; k.dt = h->g.dt;
    k.Uref = h->g.Uref; k.beta = std::fmax(0.001, 3.0/(double)p.Re); k.area = (double)(p.LX*(p.LZ - 1.0));
    k.nnodes = (double)p.NX*(double)p.NY*(double)p.NZ;
    k.drill_plane = -1;

    Ctrl c;
    std::memset(&c, 0, sizeof(c));
    c.force = h->g.force0;
    // plane sum of the initial v (what the first AccumulateUbulk sees)
    const double *dxv = nullptr, *dzv = nullptr;
    std::vector<double> dxh(p.NX), dzh(p.NZ);
    for (int x = 0; x < p.NX; x++) dxh[x] = (h->g.x[x + 4] - h->g.x[x + 2])/2.0;
    for (int z = 0; z < p.NZ; z++) dzh[z] = (h->g.z[z + 4] - h->g.z[z + 2])/2.0;
    dxv = dxh.data(); dzv = dzh.data();
    double s0 = 0.0;
    for (int z = 0; z < p.NZ; z++)
        for (int x = 0; x < p.NX; x++) {
            double r, u, v, w, f[19];
            initial_node(h, x, k.yplane, z, &r, &u, &v, &w, f);
            s0 += v*dxv[x]*dzv[z];
        }
    c.ub_slot[0] = s0;
    CK(cudaMemcpyAsync(h->ctrl, &c, sizeof(c), cudaMemcpyHostToDevice, h->stream));
    h->cur = 0;
    h->steps = 0;
    h->use_tiled = false;
    h->paired = false;
    if (p.kernel == ISLBM_KERNEL_TILED || p.kernel == ISLBM_KERNEL_AUTO || p.kernel == ISLBM_KERNEL_TILED_SINGLE) {
        int sms = 0;
        CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device));
        double wx0[7], wx2[7], wy0[7], wy2[7];
        for (int a = 0; a < 7; a++) {   // uniform spacing: the weights of the first node serve all
            wx0[a] = h->g.XP0[(size_t)a*h->g.NX6 + 3]; wx2[a] = h->g.XP2[(size_t)a*h->g.NX6 + 3];
            wy0[a] = h->g.YP0[(size_t)a*h->g.NYD6 + 3]; wy2[a] = h->g.YP2[(size_t)a*h->g.NYD6 + 3];
        }
        // the paired-node kernel where the grid allows it, else the one-node-per-thread kernel
        if (p.kernel != ISLBM_KERNEL_TILED_SINGLE && pair_supported(k, p.precision) &&
            make_pair_const(k, p.precision, wx0, wx2, wy0, wy2, sms, &h->tiled) == 0) {
            h->use_tiled = h->paired = true;
            // tensor-map plane copies unless the bulk row copies are asked for (comparison runs)
            const char *cp = std::getenv("ISLBM_PAIR_COPIES");
            if (!(cp && std::strcmp(cp, "bulk") == 0)) make_pair_maps(k, (int)h->elem, h->fbuf, &h->pmaps);
        } else if (tiled_supported(k, p.precision) && make_tiled_const(k, p.precision, wx0, wx2, wy0, wy2, sms, &h->tiled) == 0) {
            h->use_tiled = true;
        }
        if (p.kernel != ISLBM_KERNEL_AUTO && !h->use_tiled) { g_last = "tiled kernel does not support this grid"; return ISLBM_ERR_NOT_SUPPORTED; }
    }
    CK(cudaStreamSynchronize(h->stream));
    return ISLBM_OK;
}

}  // namespace

namespace islbm {
int handle_init(const islbm_params *p, islbm_handle *h) { return init_impl(p, h); }
void handle_free(islbm_handle *h) { free_handle_impl(h); }
int report_cuda(cudaError_t e, const char *what) { return cuda_fail(e, what); }
void unique_to_reference_layout(const islbm_handle *h, const double *u, double *r) { unique_to_reference(h, u, r); }
void reference_to_unique_layout(const islbm_handle *h, const double *r, double *u) { reference_to_unique(h, r, u); }
int report_status(int status, const char *msg) {
    g_last = msg;
    return status;
}
}  // namespace islbm

extern "C" {

int islbm_default_params(islbm_params *p) {
    if (!p) return ISLBM_ERR_INVALID_ARGUMENT;
    std::memset(p, 0, sizeof(*p));
    p->NX = 32; p->NY = 64; p->NZ = 48;
    p->LX = 4.5; p->LY = 9.0; p->LZ = 3.036;
    p->CFL = 0.6; p->LXi = 10.0;
    p->Re = 700.0; p->Uref = 0.05;
    p->NDTFRC = 10000;
    p->precision = ISLBM_FP64;
    p->les_cs = 0.0; p->alpha = 1.0; p->geometry = 0;
    p->init_mode = 1; p->seed = 1234ULL; p->perturb = 0.01;
    p->mass_interval = 0; p->bfl_mode = 0; p->device = 0;
    p->kernel = ISLBM_KERNEL_AUTO;
    p->hbm_budget_bytes = 0;
    return ISLBM_OK;
}

int islbm_required_bytes(const islbm_params *p, size_t *bytes) {
    if (!p || !bytes) return ISLBM_ERR_INVALID_ARGUMENT;
    const int st = validate(*p);
    if (st != ISLBM_OK) return st;
    *bytes = required_bytes(*p);
    return ISLBM_OK;
}

int islbm_init(const islbm_params *p, islbm_handle **out) {
    if (!p || !out) return ISLBM_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    islbm_handle *h = new (std::nothrow) islbm_handle();
    if (!h) return ISLBM_ERR_OUT_OF_MEMORY;
    const int st = init_impl(p, h);
    if (st != ISLBM_OK) { free_handle_impl(h); return st; }
    *out = h;
    return ISLBM_OK;
}

int islbm_step(islbm_handle *h, int nsteps) {
    if (check_handle(h) || nsteps < 0) return ISLBM_ERR_INVALID_ARGUMENT;
    CK(cudaSetDevice(h->device));
    StepLaunch L{};
    L.precision = h->p.precision;
    L.tables = h->p.precision == ISLBM_FP64 ? (const void *)&h->td : (const void *)&h->tf;
    L.k = h->k;
    L.ctrl = h->ctrl;
    L.les = h->p.les_cs > 0.0;
    L.stream = h->stream;
    L.tiled = &h->tiled;
    for (int s = 0; s < nsteps; s++) {
        const unsigned long long n = h->steps + 1;
        L.fo = h->fbuf[h->cur];
        L.fn = h->fbuf[1 - h->cur];
        L.pmaps = h->paired ? h->pmaps.for_buffer(L.fo) : nullptr;
        L.n = n;
        L.mass = h->p.mass_interval > 0 && (n % (unsigned long long)h->p.mass_interval) == 0ULL;
        L.macros_on = (s == nsteps - 1);
        for (int m = 0; m < 4; m++) L.macros[m] = h->macros[m];
        cudaError_t e = h->paired ? launch_step_pair(L) : h->use_tiled ? launch_step_tiled(L) : launch_step_gather(L);
        if (e != cudaSuccess) return cuda_fail(e, "step kernel launch");
        h->cur = 1 - h->cur;
        h->steps = n;
    }
    return ISLBM_OK;
}

int islbm_fields(islbm_handle *h, double *rho, double *u, double *v, double *w, int layout) {
    if (check_handle(h) || layout < 0 || layout > 1) return ISLBM_ERR_INVALID_ARGUMENT;
    CK(cudaSetDevice(h->device));
    double *outs[4] = {rho, u, v, w};
    for (int m = 0; m < 4; m++)
        if (outs[m]) { const int st = copy_macro(h, m, outs[m], layout); if (st) return st; }
    return ISLBM_OK;
}

int islbm_get_population(islbm_handle *h, int q, double *out, int layout) {
    if (check_handle(h) || q < 0 || q > 18 || !out || layout < 0 || layout > 1) return ISLBM_ERR_INVALID_ARGUMENT;
    CK(cudaSetDevice(h->device));
    const size_t N = h->N;
    if (layout == ISLBM_LAYOUT_UNIQUE) {
        CK(xfer_buffer(h));
        const float wq = (float)dev_ref(q);
        const void *src = (const char *)h->fbuf[h->cur] + (size_t)q*N*h->elem;
        CK(by_storage(h->p.precision, [&](auto tag) {
            using S = typename decltype(tag)::type;
            from_storage_kernel<S><<<conv_grid(N), 256, 0, h->stream>>>((const S *)src, h->xfer, N, wq);
            return cudaGetLastError();
        }));
        CK(cudaMemcpyAsync(out, h->xfer, N*8, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        return ISLBM_OK;
    }
    std::vector<char> stage(N*h->elem);
    CK(cudaMemcpyAsync(stage.data(), (const char *)h->fbuf[h->cur] + (size_t)q*N*h->elem, N*h->elem, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    std::vector<double> tmp(N);
    from_storage(h->p.precision, q, stage.data(), tmp.data(), N);
    if (layout == ISLBM_LAYOUT_REFERENCE) unique_to_reference(h, tmp.data(), out);
    else std::memcpy(out, tmp.data(), N*8);
    return ISLBM_OK;
}

int islbm_set_populations(islbm_handle *h, const double *f19, int layout) {
    if (check_handle(h) || !f19 || layout < 0 || layout > 1) return ISLBM_ERR_INVALID_ARGUMENT;
    CK(cudaSetDevice(h->device));
    const size_t N = h->N;
    const size_t nref = (size_t)(h->p.NX + 7)*(h->p.NY + 7)*(h->p.NZ + 6);
    if (layout == ISLBM_LAYOUT_UNIQUE) {
        // FP64 up, narrowed to the storage format on the device
        CK(xfer_buffer(h));
        for (int q = 0; q < 19; q++) {
            const double wq = dev_ref(q);
            CK(cudaMemcpyAsync(h->xfer, f19 + (size_t)q*N, N*8, cudaMemcpyHostToDevice, h->stream));
            void *dst = (char *)h->fbuf[h->cur] + (size_t)q*N*h->elem;
            CK(by_storage(h->p.precision, [&](auto tag) {
                using S = typename decltype(tag)::type;
                to_storage_kernel<S><<<conv_grid(N), 256, 0, h->stream>>>(h->xfer, (S *)dst, N, wq);
                return cudaGetLastError();
            }));
        }
        CK(cudaStreamSynchronize(h->stream));
        return ISLBM_OK;
    }
    std::vector<double> tmp(N);
    std::vector<char> stage(19*N*h->elem);
    for (int q = 0; q < 19; q++) {
        const double *src = layout == ISLBM_LAYOUT_REFERENCE ? f19 + (size_t)q*nref : f19 + (size_t)q*N;
        if (layout == ISLBM_LAYOUT_REFERENCE) { reference_to_unique(h, src, tmp.data()); src = tmp.data(); }
        to_storage(h->p.precision, q, src, stage.data() + (size_t)q*N*h->elem, N);
    }
    CK(cudaMemcpyAsync(h->fbuf[h->cur], stage.data(), stage.size(), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return ISLBM_OK;
}

int islbm_get_scalars(islbm_handle *h, double *force, double *rho_modify, long long *steps) {
    if (check_handle(h)) return ISLBM_ERR_INVALID_ARGUMENT;
    CK(cudaSetDevice(h->device));
    Ctrl c;
    CK(cudaMemcpyAsync(&c, h->ctrl, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (force) *force = c.force;
    if (rho_modify) *rho_modify = c.rho_modify;
    if (steps) *steps = (long long)c.step;
    return ISLBM_OK;
}

int islbm_set_force(islbm_handle *h, double force) {
    if (check_handle(h)) return ISLBM_ERR_INVALID_ARGUMENT;
    CK(cudaSetDevice(h->device));
    CK(cudaMemcpyAsync(&h->ctrl->force, &force, sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return ISLBM_OK;
}

int islbm_get_constants(islbm_handle *h, double *tau, double *niu, double *uref, double *min_size) {
    if (check_handle(h)) return ISLBM_ERR_INVALID_ARGUMENT;
    if (tau) *tau = h->g.tau;
    if (niu) *niu = h->g.niu;
    if (uref) *uref = h->g.Uref;
    if (min_size) *min_size = h->g.minSize;
    return ISLBM_OK;
}

int islbm_weight_table_bytes(islbm_handle *h, size_t *stored, size_t *per_node) {
    if (check_handle(h)) return ISLBM_ERR_INVALID_ARGUMENT;
    if (stored) *stored = h->tab_bytes;
    // per-node storage: 7 x, 7 y and 7 xi weights for each of the 18 moving directions
    if (per_node) *per_node = h->N*18*21*h->celem;
    return ISLBM_OK;
}

int islbm_get_stream(islbm_handle *h, void **stream) {
    if (check_handle(h) || !stream) return ISLBM_ERR_INVALID_ARGUMENT;
    *stream = (void *)h->stream;
    return ISLBM_OK;
}

int islbm_sync(islbm_handle *h) {
    if (check_handle(h)) return ISLBM_ERR_INVALID_ARGUMENT;
    CK(cudaSetDevice(h->device));
    CK(cudaStreamSynchronize(h->stream));
    unsigned fault = 0;
    CK(cudaMemcpy(&fault, &h->ctrl->fault, sizeof(fault), cudaMemcpyDeviceToHost));
    if (fault) { g_last = "a shared-memory pipeline wait timed out in the step kernel"; return ISLBM_ERR_CUDA; }
    return ISLBM_OK;
}

int islbm_fault_drill(islbm_handle *h, int plane) {
    if (check_handle(h) || plane < -1 || plane >= h->p.NZ) return ISLBM_ERR_INVALID_ARGUMENT;
    if (!h->use_tiled) { g_last = "the failure drill needs the tiled kernel"; return ISLBM_ERR_NOT_SUPPORTED; }
    h->k.drill_plane = plane;
    return ISLBM_OK;
}

int islbm_check_finite(islbm_handle *h, long long *bad) {
    if (check_handle(h) || !bad) return ISLBM_ERR_INVALID_ARGUMENT;
    CK(cudaSetDevice(h->device));
    Ctrl c;
    CK(cudaMemcpyAsync(&c, h->ctrl, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    *bad = c.nonfinite ? 1 : 0;
    return *bad ? ISLBM_ERR_NONFINITE : ISLBM_OK;
}

int islbm_destroy(islbm_handle *h) {
    if (!h) return ISLBM_ERR_INVALID_ARGUMENT;
    free_handle_impl(h);
    return ISLBM_OK;
}

const char *islbm_status_string(int status) {
    switch (status) {
    case ISLBM_OK: return "ok";
    case ISLBM_ERR_INVALID_ARGUMENT: return "invalid argument";
    case ISLBM_ERR_CUDA: return g_last.empty() ? "CUDA error" : g_last.c_str();
    case ISLBM_ERR_OUT_OF_MEMORY: return "out of device memory";
    case ISLBM_ERR_HBM_BUDGET: return "solve exceeds the HBM budget";
    case ISLBM_ERR_NONFINITE: return "non-finite value in the state";
    case ISLBM_ERR_NOT_SUPPORTED: return g_last.empty() ? "not supported" : g_last.c_str();
    case ISLBM_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
    }
}

int islbm_host_table(const islbm_params *p, const char *name, int idx, double *out, size_t cap, size_t *count) {
    if (!p || !name || !count) return ISLBM_ERR_INVALID_ARGUMENT;
    Geometry g;
    const int st = g.build(*p);
    if (st != ISLBM_OK) return st;
    size_t n = 0;
    const double *src = g.table(name, idx, &n);
    if (!src) return ISLBM_ERR_INVALID_ARGUMENT;
    *count = n;
    if (out) {
        if (cap < n) return ISLBM_ERR_INVALID_ARGUMENT;
        std::memcpy(out, src, n*sizeof(double));
    }
    return ISLBM_OK;
}

int islbm_host_table_int(const islbm_params *p, const char *name, int *out, size_t cap, size_t *count) {
    if (!p || !name || !count) return ISLBM_ERR_INVALID_ARGUMENT;
    Geometry g;
    const int st = g.build(*p);
    if (st != ISLBM_OK) return st;
    size_t n = 0;
    const int *src = g.table_int(name, &n);
    if (!src) return ISLBM_ERR_INVALID_ARGUMENT;
    *count = n;
    if (out) {
        if (cap < n) return ISLBM_ERR_INVALID_ARGUMENT;
        std::memcpy(out, src, n*sizeof(int));
    }
    return ISLBM_OK;
}

}  // extern "C"
