// Device state of one solve (shared by the C ABI and the serving loop).
#pragma once

#include <cuda_runtime.h>

#include "../../include/islbm.h"
#include "geometry.hpp"
#include "step_launch.hpp"
#include "step_tiled.hpp"

using namespace islbm;

struct islbm_handle {
    islbm_params p{};
    Geometry g;
    int device = 0;
    cudaStream_t stream = nullptr;
    size_t N = 0;
    size_t elem = 0;           // bytes per stored population value
    size_t celem = 0;          // bytes per compute-type value
    void *fbuf[2] = {nullptr, nullptr};
    void *macros[4] = {nullptr, nullptr, nullptr, nullptr};
    void *tabmem = nullptr;    // one allocation for all weight tables
    size_t tab_bytes = 0;
    Ctrl *ctrl = nullptr;
    Tables<double> td{};
    Tables<float> tf{};
    StepConst k{};
    int cur = 0;
    unsigned long long steps = 0;
    bool use_tiled = false;    // a tiled kernel (shared-memory tiles, TMEM ring) steps this solve
    bool paired = false;       // ... the paired-node one (step_pair.cu), else step_tiled.cu
    double *stats = nullptr;   // time-average accumulators, ISLBM_STAT_COUNT x N (allocated on first use)
    long long stats_samples = 0;
    int stats_grad = 0;        // gradient quantities requested (ISLBM_STAT_ALL sums instead of COUNT)
    int stats_nq = 0;          // quantities held by the current allocation of `stats`
    double *zslope = nullptr;  // five wall-normal derivative weights per (z, y) node

    double *xfer = nullptr;    // FP64 transfer buffer of N values for host copies (first use)
    TiledConst tiled{};
    PairMaps pmaps{};          // tensor maps of fbuf[0], fbuf[1] for the paired kernel's copies
};


namespace islbm {
// init/teardown used by the serving loop as well as islbm_init/islbm_destroy
int handle_init(const islbm_params *p, islbm_handle *h);
void handle_free(islbm_handle *h);
// record a CUDA failure for islbm_status_string and map it to a status
int report_cuda(cudaError_t e, const char *what);
// record a message for islbm_status_string and return `status`
int report_status(int status, const char *msg);
// unique [z][y][x] field -> the reference's padded layout (NYD6, NZ6, NX6)
void unique_to_reference_layout(const islbm_handle *h, const double *u, double *r);
// the reference's padded layout -> unique [z][y][x] (interior nodes)
void reference_to_unique_layout(const islbm_handle *h, const double *r, double *u);
}
