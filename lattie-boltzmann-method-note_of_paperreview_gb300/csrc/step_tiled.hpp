// Launch constants of the tiled step kernel (host-computed, passed by value).
#pragma once

#include <stddef.h>

#include <cuda.h>
#include <cuda_runtime.h>

#include "step_common.cuh"
#include "step_launch.hpp"

namespace islbm {

struct TiledConst {
    int TY;                       // streamwise rows per tile (128 / NX, 1 for NX >= 128)
    int grid;                     // persistent CTAs
    int zsegs;                    // wall-normal segments per column (work items = tiles * zsegs)
    size_t smem_bytes;            // dynamic shared memory per CTA (layout: Lay in step_tiled.cu)
    // uniform-spacing Lagrange weights as (departure - minSize, departure + minSize) pairs, the
    // operand layout of the packed FP32x2 filters: wx[a] = (wx0[a], wx2[a]), wy[b] = (wy0[b], wy2[b])
    float2 wx[7], wy[7];
    // paired-node kernel (step_pair.cu): streamwise weights as broadcast pairs (wyb[0] = (wy0, wy0),
    // wyb[1] = (wy2, wy2)) and the spanwise weights of aligned node pairs for node 0 (wxa) and
    // node 1 (wxb), set 0 = wx0, set 1 = wx2
    float2 wyb[2][7];
    float2 wxa[2][4], wxb[2][4];
    unsigned long long n;         // step number (set per launch)
};

int make_tiled_const(const StepConst &k, int precision, const double *wx0, const double *wx2, const double *wy0,
                     const double *wy2, int num_sms, TiledConst *out);

// Batched tiled step: one launch advances every solve described in `descs` by one step. Work
// items are (solve, seg*ntiles + tile): wall-normal segment seg of tile `tile`.
size_t batch_desc_bytes(int precision, int NX, bool les);
void fill_batch_desc(int precision, int NX, bool les, const Tables<float> &T, const StepConst &k, const TiledConst &tc,
                     Ctrl *ctrl, void *const macros[4], void *buf0, void *buf1, int ntiles, int nseg, void *out);
// one-time kernel attributes; call before the first launch is captured into a graph
cudaError_t prepare_step_tiled_batch(int precision, int NX, bool les);
cudaError_t launch_step_tiled_batch(int precision, int NX, bool les, const void *descs, const int2 *items, int nitems,
                                    int grid, int macros_on, cudaStream_t stream);

// Paired-node tiled step (step_pair.cu): two spanwise-adjacent nodes per thread, packed FP32x2
// arithmetic; same launch constants, the same batched interface.
bool pair_supported(const StepConst &k, int precision);
int make_pair_const(const StepConst &k, int precision, const double *wx0, const double *wx2, const double *wy0,
                    const double *wy2, int num_sms, TiledConst *out);
int pair_zsegs(int tiles, int slots, int NZ);
cudaError_t launch_step_pair(const StepLaunch &L);
// Tensor maps of a solve's two population buffers for the paired kernel's plane copies, one per
// box shape (m[b][j]: buffer buf[b]; box j = NX x (TY + 6) rows x 2 or 4 populations, NX x TY
// rows x 2 or 4 populations); ok is false where they are not used (NX > 256, or the driver refused
// them), and the kernel then copies row runs with cp.async.bulk. A launch takes the maps whose
// buffer it reads (`for_buffer`), so swapping a handle's buffers cannot pair a map with the
// wrong one.
struct PairMaps {
    CUtensorMap m[2][4];
    const void *buf[2] = {nullptr, nullptr};
    bool ok = false;
    const void *for_buffer(const void *fo) const {
        for (int b = 0; b < 2; b++)
            if (ok && buf[b] == fo) return (const void *)m[b];
        return nullptr;
    }
};
bool make_pair_maps(const StepConst &k, int elem_bytes, void *const buf[2], PairMaps *out);
size_t pair_batch_desc_bytes(int precision, int NX, bool les);
void fill_pair_batch_desc(int precision, int NX, bool les, const Tables<float> &T, const StepConst &k, const TiledConst &tc,
                          Ctrl *ctrl, void *const macros[4], void *buf0, void *buf1, int ntiles, int nseg, void *out);
cudaError_t prepare_step_pair_batch(int precision, int NX, bool les);
cudaError_t launch_step_pair_batch(int precision, int NX, bool les, const void *descs, const int2 *items, int nitems,
                                   int grid, int macros_on, cudaStream_t stream);

}  // namespace islbm
