// Whole-field diagnostics of a solve, computed from its current populations.
//
// The reference checks the total mass every 100 steps by copying all populations to the host
// (main loop around SendDataToCPU, C/communication.h:260-273) and, in Monitor.dat
// (C/monitor.h:4-26), records the velocity at one probe with the body force. Here one
// reduction over the unique nodes gives, in FP64:
//   out[0]  total mass        sum rho
//   out[1]  mean momentum     sum rho*v / N   (streamwise, the bulk-flow direction)
//   out[2]  kinetic energy    sum rho*|u|^2 / 2
//   out[3]  maximum speed     max |u|
// with rho = sum_q f_q and rho*u = sum_q e_q f_q, the moments of C/evolution.h:600-607.
//
// Reduction: blocks of 256 threads each take a contiguous run of DIAG_NODES_PER_BLOCK nodes,
// reduce it in FP64 and write one partial record to scratch; the last block to finish (a
// done counter in scratch, which must be zero at launch) adds the records in block order, so
// the result does not depend on scheduling, and writes it to scratch.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>

#include "handle.hpp"

namespace islbm {
namespace {

constexpr int DIAG_THREADS = 256;
constexpr int DIAG_PER_THREAD = 8;
constexpr size_t DIAG_NODES_PER_BLOCK = (size_t)DIAG_THREADS*DIAG_PER_THREAD;
// scratch layout in bytes: [0, 256) done counter; [256, 512) result (4 doubles);
// [512, 512 + 32*blocks) partial records (4 doubles per block)
constexpr size_t DIAG_RESULT_OFF = 256, DIAG_PARTIAL_OFF = 512;

size_t diag_blocks(size_t n) { return (n + DIAG_NODES_PER_BLOCK - 1)/DIAG_NODES_PER_BLOCK; }
size_t diag_scratch_bytes(size_t n) { return DIAG_PARTIAL_OFF + 32*diag_blocks(n); }

template <class S>
__global__ void __launch_bounds__(DIAG_THREADS) diag_kernel(const S *__restrict__ f, size_t n, unsigned char *scratch) {
    using C = typename Storage<S>::C;
    unsigned *done = (unsigned *)scratch;
    double *result = (double *)(scratch + DIAG_RESULT_OFF);
    double *part = (double *)(scratch + DIAG_PARTIAL_OFF);
    double m = 0.0, mv = 0.0, ke = 0.0, vmax = 0.0;
    const size_t first = (size_t)blockIdx.x*DIAG_NODES_PER_BLOCK;
#pragma unroll 1
    for (int r = 0; r < DIAG_PER_THREAD; r++) {
        const size_t i = first + (size_t)r*DIAG_THREADS + threadIdx.x;
        if (i >= n) break;
        C F[19];
#pragma unroll
        for (int q = 0; q < 19; q++) F[q] = load_f<S>(f + (size_t)q*n, i, q);
        double rho = 0.0;
#pragma unroll
        for (int q = 0; q < 19; q++) rho += (double)F[q];
        const double ju = (double)F[1] + F[7] + F[9] + F[11] + F[13] - ((double)F[2] + F[8] + F[10] + F[12] + F[14]);
        const double jv = (double)F[3] + F[7] + F[8] + F[15] + F[17] - ((double)F[4] + F[9] + F[10] + F[16] + F[18]);
        const double jw = (double)F[5] + F[11] + F[12] + F[15] + F[16] - ((double)F[6] + F[13] + F[14] + F[17] + F[18]);
        const double u2 = (ju*ju + jv*jv + jw*jw)/(rho*rho);
        m += rho;
        mv += jv;
        ke += 0.5*rho*u2;
        vmax = fmax(vmax, sqrt(u2));
        if (!(u2 == u2)) vmax = u2;   // keep a NaN visible (fmax drops it)
    }
    __shared__ double red[4][DIAG_THREADS/32];
    __shared__ bool last;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        m += __shfl_down_sync(0xffffffffu, m, o);
        mv += __shfl_down_sync(0xffffffffu, mv, o);
        ke += __shfl_down_sync(0xffffffffu, ke, o);
        const double other = __shfl_down_sync(0xffffffffu, vmax, o);
        vmax = (other == other) ? fmax(vmax, other) : other;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { red[0][warp] = m; red[1][warp] = mv; red[2][warp] = ke; red[3][warp] = vmax; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
        for (int w = 0; w < DIAG_THREADS/32; w++) {
            s0 += red[0][w]; s1 += red[1][w]; s2 += red[2][w];
            s3 = (red[3][w] == red[3][w]) ? fmax(s3, red[3][w]) : red[3][w];
        }
        double *rec = part + 4*(size_t)blockIdx.x;
        rec[0] = s0; rec[1] = s1; rec[2] = s2; rec[3] = s3;
        __threadfence();
        last = atomicAdd(done, 1u) == gridDim.x - 1u;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
        for (unsigned b = 0; b < gridDim.x; b++) {
            const double *rec = part + 4*(size_t)b;
            s0 += __ldcg(rec); s1 += __ldcg(rec + 1); s2 += __ldcg(rec + 2);
            const double v = __ldcg(rec + 3);
            s3 = (v == v) ? fmax(s3, v) : v;
        }
        result[0] = s0;
        result[1] = s1/(double)n;
        result[2] = s2;
        result[3] = s3;
        *done = 0u;
    }
}

cudaError_t launch_diag(const islbm_handle *h, unsigned char *scratch, cudaStream_t st) {
    const void *f = h->fbuf[h->cur];
    const unsigned grid = (unsigned)diag_blocks(h->N);
    switch (h->p.precision) {
    case ISLBM_FP64: diag_kernel<double><<<grid, DIAG_THREADS, 0, st>>>((const double *)f, h->N, scratch); break;
    case ISLBM_FP32: diag_kernel<float><<<grid, DIAG_THREADS, 0, st>>>((const float *)f, h->N, scratch); break;
    case ISLBM_FP16_DEV: diag_kernel<__half><<<grid, DIAG_THREADS, 0, st>>>((const __half *)f, h->N, scratch); break;
    default:
        diag_kernel<__nv_bfloat16><<<grid, DIAG_THREADS, 0, st>>>((const __nv_bfloat16 *)f, h->N, scratch);
        break;
    }
    return cudaGetLastError();
}

// Limits of islbm_diagnostics_noalloc: DIAG_NOALLOC_MAX_BLOCKS reduction blocks of 2048 nodes.
constexpr size_t DIAG_NOALLOC_MAX_BLOCKS = 16384;
constexpr size_t DIAG_NOALLOC_MAX_NODES = DIAG_NOALLOC_MAX_BLOCKS*DIAG_NODES_PER_BLOCK;   // 33,554,432
constexpr size_t DIAG_NOALLOC_BYTES = DIAG_PARTIAL_OFF + 32*DIAG_NOALLOC_MAX_BLOCKS;      // 524,800
constexpr int DIAG_MAX_DEVICES = 64;

}  // namespace
}  // namespace islbm

// Scratch of islbm_diagnostics_noalloc: one fixed array in device memory (one copy per device).
static __device__ __align__(256) unsigned char g_diag_scratch[islbm::DIAG_NOALLOC_BYTES];

// Device address of g_diag_scratch per device: in host code the symbol name is not a device
// address, so it is looked up once per device, with that device current. The address is kept
// for the life of the process; a call checks that it still names device memory of that device
// (a host program that called cudaDeviceReset has a new context, in which the module and its
// array are loaded again) and looks it up again when it does not.
static std::mutex g_diag_mu;
static unsigned char *g_diag_ptr[islbm::DIAG_MAX_DEVICES] = {};

using namespace islbm;

extern "C" int islbm_diagnostics(islbm_handle *h, double *out) {
    if (!h || !out) return ISLBM_ERR_INVALID_ARGUMENT;
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return report_cuda(e, "cudaSetDevice");
    unsigned char *scratch = nullptr;
    e = cudaMalloc(&scratch, diag_scratch_bytes(h->N));
    if (e != cudaSuccess) return report_cuda(e, "cudaMalloc(diagnostics scratch)");
    e = cudaMemsetAsync(scratch, 0, DIAG_RESULT_OFF, h->stream);   // the done counter starts at zero
    if (e == cudaSuccess) e = launch_diag(h, scratch, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, scratch + DIAG_RESULT_OFF, 4*sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    const cudaError_t ef = cudaFree(scratch);
    if (e != cudaSuccess) return report_cuda(e, "diagnostics");
    if (ef != cudaSuccess) return report_cuda(ef, "cudaFree(diagnostics scratch)");
    return ISLBM_OK;
}

// No-allocation variant of islbm_diagnostics: the same kernel on a fixed scratch array.
extern "C" int islbm_diagnostics_noalloc(islbm_handle *h, double *out) {
    if (!h || !out) return ISLBM_ERR_INVALID_ARGUMENT;
    if (h->N > DIAG_NOALLOC_MAX_NODES) {
        const std::string msg = "islbm_diagnostics_noalloc: the grid has " + std::to_string(h->N) +
                                " nodes; its fixed scratch holds at most " + std::to_string(DIAG_NOALLOC_MAX_NODES) +
                                " (use islbm_diagnostics)";
        return report_status(ISLBM_ERR_NOT_SUPPORTED, msg.c_str());
    }
    if (h->device < 0 || h->device >= DIAG_MAX_DEVICES) return report_status(ISLBM_ERR_NOT_SUPPORTED, "device index too large");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return report_cuda(e, "cudaSetDevice");
    unsigned char *scratch = nullptr;
    {
        // set-up on the first call on this device, with the device current
        std::lock_guard<std::mutex> lock(g_diag_mu);
        if (g_diag_ptr[h->device]) {
            cudaPointerAttributes a;
            if (cudaPointerGetAttributes(&a, g_diag_ptr[h->device]) != cudaSuccess || a.type != cudaMemoryTypeDevice ||
                a.device != h->device) {
                (void)cudaGetLastError();
                g_diag_ptr[h->device] = nullptr;
            }
        }
        if (!g_diag_ptr[h->device]) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_diag_scratch);
            if (e != cudaSuccess) return report_cuda(e, "cudaGetSymbolAddress(diagnostics scratch)");
            g_diag_ptr[h->device] = (unsigned char *)p;
        }
        scratch = g_diag_ptr[h->device];
    }
    e = cudaMemsetAsync(scratch, 0, DIAG_RESULT_OFF, h->stream);   // the done counter starts at zero
    if (e == cudaSuccess) e = launch_diag(h, scratch, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, scratch + DIAG_RESULT_OFF, 4*sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return report_cuda(e, "diagnostics (no allocation)");
    return ISLBM_OK;
}
