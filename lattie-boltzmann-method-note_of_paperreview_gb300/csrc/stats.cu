// Time-averaged turbulence statistics of a solve (MeanVars, C/statistics.h:122-174).
//
// Per unique node, FP64 sums over samples of the 24 quantities of the reference, in its order:
//   U V W P, UU UV UW VV VW WW, PU PV PW PP, KT, UUU UUV UUW VVU VVV VVW WWU WWV WWW
// with P = rho/3 - 1/3 and KT = (u^2 + v^2 + w^2)/2, taken from the macroscopic fields of the
// last step (islbm_step writes them on its last step). The accumulators are one allocation of
// 24*N doubles, laid out [quantity][z][y][x]; a sample reads 16 B (FP32 fields) or 32 B (FP64)
// and updates 24 x 8 B per node, so it is HBM bound at about 400 B per node.
#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "handle.hpp"

namespace islbm {
namespace {

template <class C>
__global__ void stats_kernel(const C *__restrict__ rho, const C *__restrict__ u, const C *__restrict__ v,
                             const C *__restrict__ w, double *__restrict__ acc, size_t n) {
    for (size_t i = blockIdx.x*(size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x*blockDim.x) {
        const double u1 = (double)u[i], v1 = (double)v[i], w1 = (double)w[i];
        const double p1 = 1.0/3.0*(double)rho[i] - 1.0/3.0;
        double *a = acc + i;
        // same products as the reference accumulates (C/statistics.h:145-172)
        a[0*n] += u1; a[1*n] += v1; a[2*n] += w1; a[3*n] += p1;
        a[4*n] += u1*u1; a[5*n] += u1*v1; a[6*n] += u1*w1; a[7*n] += v1*v1; a[8*n] += v1*w1; a[9*n] += w1*w1;
        a[10*n] += p1*u1; a[11*n] += p1*v1; a[12*n] += p1*w1; a[13*n] += p1*p1;
        a[14*n] += 0.5*(u1*u1 + v1*v1 + w1*w1);
        a[15*n] += u1*u1*u1; a[16*n] += u1*u1*v1; a[17*n] += u1*u1*w1;
        a[18*n] += v1*v1*u1; a[19*n] += v1*v1*v1; a[20*n] += v1*v1*w1;
        a[21*n] += w1*w1*u1; a[22*n] += w1*w1*v1; a[23*n] += w1*w1*w1;
    }
}

// Squared velocity gradients of MeanVars' companion (MeanDerivatives, C/statistics.h:176-222):
// x and y by the fourth-order central difference (8 (f[+1] - f[-1]) - (f[+2] - f[-2])) / 12 / h,
// periodic; z by five weights per node over the nodes n .. n + 4 of its column,
// n = clamp(z - 2, 0, NZ - 5).
template <class C>
__global__ void grad_kernel(const C *__restrict__ u, const C *__restrict__ v, const C *__restrict__ w,
                            const double *__restrict__ zs, double *__restrict__ acc, int NX, int NY, int NZ, double dx,
                            double dy) {
    const size_t n = (size_t)NX*NY*NZ;
    for (size_t i = blockIdx.x*(size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x*blockDim.x) {
        const int x = (int)(i % NX);
        const int y = (int)((i/NX) % NY);
        const int z = (int)(i/((size_t)NX*NY));
        const size_t row = i - x, plane = (size_t)NX*NY;
        const size_t col = i - (size_t)y*NX;   // (x, 0, z)
        auto ddx = [&](const C *f) {
            const double a = f[row + ((x + 1) % NX)] - (double)f[row + ((x - 1 + NX) % NX)];
            const double b = f[row + ((x + 2) % NX)] - (double)f[row + ((x - 2 + NX) % NX)];
            return (8.0*a - b)/12.0/dx;
        };
        auto ddy = [&](const C *f) {
            const double a = f[col + (size_t)((y + 1) % NY)*NX] - (double)f[col + (size_t)((y - 1 + NY) % NY)*NX];
            const double b = f[col + (size_t)((y + 2) % NY)*NX] - (double)f[col + (size_t)((y - 2 + NY) % NY)*NX];
            return (8.0*a - b)/12.0/dy;
        };
        const int nb = min(max(z - 2, 0), NZ - 5);
        const double *c = zs + ((size_t)z*NY + y)*5;
        auto ddz = [&](const C *f) {
            const size_t b0 = (size_t)nb*plane + (size_t)y*NX + x;
            double s = 0.0;
            for (int m = 0; m < 5; m++) s += c[m]*(double)f[b0 + (size_t)m*plane];
            return s;
        };
        const double g[9] = {ddx(u), ddy(u), ddz(u), ddx(v), ddy(v), ddz(v), ddx(w), ddy(w), ddz(w)};
#pragma unroll
        for (int q = 0; q < 9; q++) acc[(size_t)(ISLBM_STAT_DUDX2 + q)*n + i] += g[q]*g[q];
    }
}

// derivative at t of the Lagrange polynomial through the five nodes zn, weight of node m
double lagrange_slope(const double *zn, int m, double t) {
    double s = 0.0;
    for (int l = 0; l < 5; l++) {
        if (l == m) continue;
        double p = 1.0/(zn[m] - zn[l]);
        for (int i = 0; i < 5; i++)
            if (i != m && i != l) p *= (t - zn[i])/(zn[m] - zn[i]);
        s += p;
    }
    return s;
}

}  // namespace
}  // namespace islbm

using namespace islbm;

extern "C" int islbm_stats_gradients(islbm_handle *h, int on) {
    if (!h || on < 0 || on > 1) return ISLBM_ERR_INVALID_ARGUMENT;
    if (h->p.NZ < 5) return report_status(ISLBM_ERR_NOT_SUPPORTED, "gradient statistics need NZ >= 5");
    h->stats_grad = on;
    if (on && !h->zslope) {
        const Geometry &g = h->g;
        const int NY = h->p.NY, NZ = h->p.NZ;
        std::vector<double> w((size_t)NZ*NY*5);
        for (int z = 0; z < NZ; z++)
            for (int y = 0; y < NY; y++) {
                const int j = y + 3, nb = std::min(std::max(z - 2, 0), NZ - 5);
                double zn[5];
                for (int m = 0; m < 5; m++) zn[m] = g.z[(size_t)j*g.NZ6 + 3 + nb + m];
                const double t = g.z[(size_t)j*g.NZ6 + 3 + z];
                for (int m = 0; m < 5; m++) w[((size_t)z*NY + y)*5 + m] = lagrange_slope(zn, m, t);
            }
        cudaError_t e = cudaSetDevice(h->device);
        if (e == cudaSuccess) e = cudaMalloc(&h->zslope, w.size()*sizeof(double));
        if (e == cudaSuccess) e = cudaMemcpy(h->zslope, w.data(), w.size()*sizeof(double), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return report_cuda(e, "gradient weights");
    }
    return ISLBM_OK;
}

extern "C" {

int islbm_stats_reset(islbm_handle *h) {
    if (!h) return ISLBM_ERR_INVALID_ARGUMENT;
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return report_cuda(e, "cudaSetDevice");
    const int nq = h->stats_grad ? ISLBM_STAT_ALL : ISLBM_STAT_COUNT;
    const size_t bytes = (size_t)nq*h->N*sizeof(double);
    if (h->stats && h->stats_nq != nq) { cudaFree(h->stats); h->stats = nullptr; }
    if (!h->stats) {
        e = cudaMalloc(&h->stats, bytes);
        if (e != cudaSuccess) { h->stats = nullptr; return report_cuda(e, "cudaMalloc(statistics)"); }
        h->stats_nq = nq;
    }
    e = cudaMemsetAsync(h->stats, 0, bytes, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return report_cuda(e, "statistics reset");
    h->stats_samples = 0;
    return ISLBM_OK;
}

int islbm_stats_accumulate(islbm_handle *h) {
    if (!h) return ISLBM_ERR_INVALID_ARGUMENT;
    if (!h->stats) {
        const int st = islbm_stats_reset(h);
        if (st != ISLBM_OK) return st;
    }
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return report_cuda(e, "cudaSetDevice");
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
    if (e != cudaSuccess) return report_cuda(e, "cudaDeviceGetAttribute");
    const unsigned grid = (unsigned)std::min<size_t>((size_t)sms*8, (h->N + 255)/256);
    if (h->celem == 8)
        stats_kernel<double><<<grid, 256, 0, h->stream>>>((const double *)h->macros[0], (const double *)h->macros[1],
                                                          (const double *)h->macros[2], (const double *)h->macros[3],
                                                          h->stats, h->N);
    else
        stats_kernel<float><<<grid, 256, 0, h->stream>>>((const float *)h->macros[0], (const float *)h->macros[1],
                                                         (const float *)h->macros[2], (const float *)h->macros[3],
                                                         h->stats, h->N);
    e = cudaGetLastError();
    if (e == cudaSuccess && h->stats_nq == ISLBM_STAT_ALL) {
        const double dx = h->p.LX/h->p.NX, dy = h->p.LY/h->p.NY;
        if (h->celem == 8)
            grad_kernel<double><<<grid, 256, 0, h->stream>>>((const double *)h->macros[1], (const double *)h->macros[2],
                                                             (const double *)h->macros[3], h->zslope, h->stats,
                                                             h->p.NX, h->p.NY, h->p.NZ, dx, dy);
        else
            grad_kernel<float><<<grid, 256, 0, h->stream>>>((const float *)h->macros[1], (const float *)h->macros[2],
                                                            (const float *)h->macros[3], h->zslope, h->stats,
                                                            h->p.NX, h->p.NY, h->p.NZ, dx, dy);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return report_cuda(e, "statistics kernel launch");
    h->stats_samples++;
    return ISLBM_OK;
}

int islbm_stats_samples(islbm_handle *h, long long *samples) {
    if (!h || !samples) return ISLBM_ERR_INVALID_ARGUMENT;
    *samples = h->stats_samples;
    return ISLBM_OK;
}

int islbm_stats_mean(islbm_handle *h, int quantity, double *out, int layout) {
    if (!h || !out || quantity < 0 || quantity >= (h->stats ? h->stats_nq : 0) || layout < 0 || layout > 1)
        return ISLBM_ERR_INVALID_ARGUMENT;
    if (!h->stats || h->stats_samples == 0) return report_status(ISLBM_ERR_NOT_SUPPORTED, "no statistics samples");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return report_cuda(e, "cudaSetDevice");
    std::vector<double> sum(h->N);
    e = cudaMemcpyAsync(sum.data(), h->stats + (size_t)quantity*h->N, h->N*sizeof(double), cudaMemcpyDeviceToHost,
                        h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return report_cuda(e, "statistics read");
    const double inv = 1.0/(double)h->stats_samples;
    for (size_t i = 0; i < h->N; i++) sum[i] *= inv;
    if (layout == ISLBM_LAYOUT_REFERENCE) unique_to_reference_layout(h, sum.data(), out);
    else std::memcpy(out, sum.data(), h->N*sizeof(double));
    return ISLBM_OK;
}

int islbm_stats_profile(islbm_handle *h, int quantity, int y, double *out) {
    if (!h || !out || quantity < 0 || quantity >= (h->stats ? h->stats_nq : 0) || y < 0 || y >= h->p.NY)
        return ISLBM_ERR_INVALID_ARGUMENT;
    if (!h->stats || h->stats_samples == 0) return report_status(ISLBM_ERR_NOT_SUPPORTED, "no statistics samples");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return report_cuda(e, "cudaSetDevice");
    const int NX = h->p.NX, NY = h->p.NY, NZ = h->p.NZ;
    std::vector<double> slab((size_t)NX*NZ);
    // the (z, x) slab of streamwise row y: NZ rows of NX values, NY*NX apart
    e = cudaMemcpy2DAsync(slab.data(), NX*sizeof(double), h->stats + (size_t)quantity*h->N + (size_t)y*NX,
                          (size_t)NY*NX*sizeof(double), NX*sizeof(double), NZ, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return report_cuda(e, "statistics profile read");
    const double inv = 1.0/((double)h->stats_samples*NX);
    for (int z = 0; z < NZ; z++) {
        double s = 0.0;
        for (int x = 0; x < NX; x++) s += slab[(size_t)z*NX + x];
        out[z] = s*inv;
    }
    return ISLBM_OK;
}

int islbm_stats_wall_shear(islbm_handle *h, double *cf) {
    if (!h || !cf) return ISLBM_ERR_INVALID_ARGUMENT;
    if (!h->stats || h->stats_samples == 0) return report_status(ISLBM_ERR_NOT_SUPPORTED, "no statistics samples");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return report_cuda(e, "cudaSetDevice");
    const int NX = h->p.NX, NY = h->p.NY;
    const size_t plane = (size_t)NX*NY;
    // the two lowest planes (z = 0, 1) of the time sums of V and W
    std::vector<double> v(2*plane), w(2*plane);
    e = cudaMemcpyAsync(v.data(), h->stats + (size_t)ISLBM_STAT_V*h->N, 2*plane*sizeof(double), cudaMemcpyDeviceToHost,
                        h->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(w.data(), h->stats + (size_t)ISLBM_STAT_W*h->N, 2*plane*sizeof(double),
                            cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return report_cuda(e, "statistics wall read");
    const Geometry &g = h->g;
    const double inv = 1.0/((double)h->stats_samples*NX);
    for (int y = 0; y < NY; y++) {
        const int j = y + 3;
        // wall height z_h[j*NZ6 + 2] and its streamwise slope (central difference, periodic rows)
        const double zw = g.z[(size_t)j*g.NZ6 + 2];
        const double zm = g.z[(size_t)(j - 1)*g.NZ6 + 2], zp = g.z[(size_t)(j + 1)*g.NZ6 + 2];
        const double slope = (zp - zm)/(g.y[j + 1] - g.y[j - 1]);
        const double norm = std::sqrt(1.0 + slope*slope);
        double ut[2], d[2];
        for (int k = 0; k < 2; k++) {
            double sv = 0.0, sw = 0.0;
            for (int x = 0; x < NX; x++) { sv += v[(size_t)k*plane + (size_t)y*NX + x]; sw += w[(size_t)k*plane + (size_t)y*NX + x]; }
            ut[k] = (sv*inv + slope*sw*inv)/norm;                       // tangential mean velocity
            d[k] = (g.z[(size_t)j*g.NZ6 + 3 + k] - zw)/norm;            // distance from the wall
        }
        // u(d) = a d + b d^2 through the wall (u = 0) and the two lowest nodes
        const double a = (ut[0]*d[1]*d[1] - ut[1]*d[0]*d[0])/(d[0]*d[1]*(d[1] - d[0]));
        cf[y] = 2.0*g.niu*a/(g.Uref*g.Uref);
    }
    return ISLBM_OK;
}


// Statistics files of the reference (Launch_OutputTB / OutputTBData and InitialTBUsingBkpData /
// ReadTBData, C/fileIO.h:356-500): <dir>/accu.dat holds the sample count as text ("%d"), and each
// quantity's running sum is <dir>/<NAME>/<NAME>_<rank>.bin, raw FP64 in the order
// k = 3..NZ6-4, j = 3..NYD6-4, i = 3..NX6-4 of the padded layout (NZ x (NY+1) x (NX+1) values:
// the periodic end nodes j = NY+3, i = NX+3 are written as copies of j = 3, i = 3).
static const char *const kStatNames[ISLBM_STAT_ALL] = {
    "U", "V", "W", "P", "UU", "UV", "UW", "VV", "VW", "WW", "PU", "PV", "PW", "PP", "KT",
    "UUU", "UUV", "UUW", "VVU", "VVV", "VVW", "WWU", "WWV", "WWW",
    "DUDX2", "DUDY2", "DUDZ2", "DVDX2", "DVDY2", "DVDZ2", "DWDX2", "DWDY2", "DWDZ2"};

static std::string tb_path(const char *dir, int q, int rank) {
    return std::string(dir) + "/" + kStatNames[q] + "/" + kStatNames[q] + "_" + std::to_string(rank) + ".bin";
}

int islbm_stats_write(islbm_handle *h, const char *dir, int rank) {
    if (!h || !dir) return ISLBM_ERR_INVALID_ARGUMENT;
    if (!h->stats) return report_status(ISLBM_ERR_NOT_SUPPORTED, "no statistics to write (islbm_stats_reset first)");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return report_cuda(e, "cudaSetDevice");
    const int NX = h->p.NX, NY = h->p.NY, NZ = h->p.NZ;
    {
        const std::string path = std::string(dir) + "/accu.dat";
        FILE *fp = std::fopen(path.c_str(), "w");
        if (!fp) return report_status(ISLBM_ERR_INVALID_ARGUMENT, ("cannot write " + path).c_str());
        std::fprintf(fp, "%lld", h->stats_samples);
        if (std::fclose(fp) != 0) return report_status(ISLBM_ERR_INVALID_ARGUMENT, ("cannot write " + path).c_str());
    }
    std::vector<double> sum(h->N), out((size_t)NZ*(NY + 1)*(NX + 1));
    for (int q = 0; q < h->stats_nq; q++) {
        e = cudaMemcpyAsync(sum.data(), h->stats + (size_t)q*h->N, h->N*sizeof(double), cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) return report_cuda(e, "statistics read");
        size_t o = 0;
        for (int z = 0; z < NZ; z++)
            for (int j = 0; j <= NY; j++)
                for (int i = 0; i <= NX; i++) out[o++] = sum[((size_t)z*NY + (j % NY))*NX + (i % NX)];
        const std::string sub = std::string(dir) + "/" + kStatNames[q];
        if (mkdir(sub.c_str(), 0755) != 0 && errno != EEXIST)
            return report_status(ISLBM_ERR_INVALID_ARGUMENT, ("cannot create " + sub).c_str());
        const std::string path = tb_path(dir, q, rank);
        FILE *fp = std::fopen(path.c_str(), "wb");
        if (!fp) return report_status(ISLBM_ERR_INVALID_ARGUMENT, ("cannot write " + path).c_str());
        const size_t w = std::fwrite(out.data(), sizeof(double), out.size(), fp);
        if (std::fclose(fp) != 0 || w != out.size()) return report_status(ISLBM_ERR_INVALID_ARGUMENT, ("short write " + path).c_str());
    }
    return ISLBM_OK;
}

int islbm_stats_read(islbm_handle *h, const char *dir, int rank) {
    if (!h || !dir) return ISLBM_ERR_INVALID_ARGUMENT;
    long long samples = 0;
    {
        const std::string path = std::string(dir) + "/accu.dat";
        FILE *fp = std::fopen(path.c_str(), "r");
        if (!fp) return report_status(ISLBM_ERR_INVALID_ARGUMENT, ("cannot read " + path).c_str());
        const int got = std::fscanf(fp, "%lld", &samples);
        std::fclose(fp);
        if (got != 1 || samples < 0) return report_status(ISLBM_ERR_INVALID_ARGUMENT, ("bad sample count in " + path).c_str());
    }
    int st = islbm_stats_reset(h);   // allocates (gradients as enabled) and zeroes the sums
    if (st != ISLBM_OK) return st;
    const int NX = h->p.NX, NY = h->p.NY, NZ = h->p.NZ;
    std::vector<double> in((size_t)NZ*(NY + 1)*(NX + 1)), sum(h->N);
    for (int q = 0; q < h->stats_nq; q++) {
        const std::string path = tb_path(dir, q, rank);
        FILE *fp = std::fopen(path.c_str(), "rb");
        if (!fp) return report_status(ISLBM_ERR_INVALID_ARGUMENT, ("cannot read " + path).c_str());
        const size_t r = std::fread(in.data(), sizeof(double), in.size(), fp);
        std::fclose(fp);
        if (r != in.size()) return report_status(ISLBM_ERR_INVALID_ARGUMENT, ("short file " + path).c_str());
        for (int z = 0; z < NZ; z++)
            for (int j = 0; j < NY; j++)
                for (int i = 0; i < NX; i++)
                    sum[((size_t)z*NY + j)*NX + i] = in[((size_t)z*(NY + 1) + j)*(NX + 1) + i];
        cudaError_t e = cudaMemcpyAsync(h->stats + (size_t)q*h->N, sum.data(), h->N*sizeof(double), cudaMemcpyHostToDevice,
                                        h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) return report_cuda(e, "statistics upload");
    }
    h->stats_samples = samples;
    return ISLBM_OK;
}

}  // extern "C"
