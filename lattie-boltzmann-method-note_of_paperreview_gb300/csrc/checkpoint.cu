// Checkpoint / restart in the reference's file format.
//
// The reference writes, per rank, raw FP64 arrays of NX6*NZ6*NYD6 values in its padded layout
// (OutputData, C/fileIO.h:52-67): rho, u, v, w and f0..f18 as <dir>/<name>_<rank>.bin, plus the
// body force as text in <dir>/0_force.dat ("%.15lf", C/fileIO.h:262-266), and reads them back in
// InitialUsingBkpData (C/fileIO.h:298-354). The same files are written and read here, so a run
// of either code can be resumed by the other. The text force keeps 15 decimals; to resume a run
// of this library exactly, the controller state (force, bulk-velocity window, step counter) is
// also written as <dir>/islbm_ctrl_<rank>.bin and used when present.
#include <sys/stat.h>

#include <cerrno>
#include <cstdio>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "handle.hpp"

namespace {

const char *const kMacroNames[4] = {"rho", "u", "v", "w"};

std::string path_of(const char *dir, const std::string &name, int rank) {
    return std::string(dir) + "/" + name + "_" + std::to_string(rank) + ".bin";
}

int write_raw(const std::string &path, const double *data, size_t n) {
    FILE *fp = std::fopen(path.c_str(), "wb");
    if (!fp) return islbm::report_status(ISLBM_ERR_INVALID_ARGUMENT, ("cannot write " + path).c_str());
    const size_t w = std::fwrite(data, sizeof(double), n, fp);
    const int closed = std::fclose(fp);
    if (w != n || closed != 0) return islbm::report_status(ISLBM_ERR_INVALID_ARGUMENT, ("short write " + path).c_str());
    return ISLBM_OK;
}

int read_raw(const std::string &path, double *data, size_t n) {
    FILE *fp = std::fopen(path.c_str(), "rb");
    if (!fp) return islbm::report_status(ISLBM_ERR_INVALID_ARGUMENT, ("cannot read " + path).c_str());
    const size_t r = std::fread(data, sizeof(double), n, fp);
    std::fclose(fp);
    if (r != n) return islbm::report_status(ISLBM_ERR_INVALID_ARGUMENT, ("short file " + path).c_str());
    return ISLBM_OK;
}

struct CtrlFile {
    char magic[8];               // "ISLBMCK1"
    unsigned long long steps;
    int cur;
    int pad;
    islbm::Ctrl ctrl;
};

}  // namespace

using namespace islbm;

extern "C" {

int islbm_checkpoint_write(islbm_handle *h, const char *dir, int rank) {
    if (!h || !dir) return ISLBM_ERR_INVALID_ARGUMENT;
    const size_t nref = (size_t)(h->p.NX + 7)*(h->p.NY + 7)*(h->p.NZ + 6);
    std::vector<double> buf(nref);
    for (int q = 0; q < 19; q++) {
        int st = islbm_get_population(h, q, buf.data(), ISLBM_LAYOUT_REFERENCE);
        if (st == ISLBM_OK) st = write_raw(path_of(dir, "f" + std::to_string(q), rank), buf.data(), nref);
        if (st != ISLBM_OK) return st;
    }
    for (int m = 0; m < 4; m++) {
        double *outs[4] = {nullptr, nullptr, nullptr, nullptr};
        outs[m] = buf.data();
        int st = islbm_fields(h, outs[0], outs[1], outs[2], outs[3], ISLBM_LAYOUT_REFERENCE);
        if (st == ISLBM_OK) st = write_raw(path_of(dir, kMacroNames[m], rank), buf.data(), nref);
        if (st != ISLBM_OK) return st;
    }
    CtrlFile cf{};
    std::memcpy(cf.magic, "ISLBMCK1", 8);
    cf.steps = h->steps;
    cf.cur = 0;
    cudaError_t e = cudaSetDevice(h->device);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&cf.ctrl, h->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return report_cuda(e, "checkpoint controller read");
    // the reference's force file
    const std::string fpath = std::string(dir) + "/0_force.dat";
    FILE *fp = std::fopen(fpath.c_str(), "w");
    if (!fp) return report_status(ISLBM_ERR_INVALID_ARGUMENT, ("cannot write " + fpath).c_str());
    std::fprintf(fp, "%.15lf", cf.ctrl.force);
    std::fclose(fp);
    const std::string cpath = std::string(dir) + "/islbm_ctrl_" + std::to_string(rank) + ".bin";
    fp = std::fopen(cpath.c_str(), "wb");
    if (!fp) return report_status(ISLBM_ERR_INVALID_ARGUMENT, ("cannot write " + cpath).c_str());
    const size_t w = std::fwrite(&cf, sizeof(cf), 1, fp);
    if (std::fclose(fp) != 0 || w != 1) return report_status(ISLBM_ERR_INVALID_ARGUMENT, ("short write " + cpath).c_str());
    if (h->stats) {   // the running statistics, in the reference's statistics files
        const std::string sdir = std::string(dir) + "/statistics";
        if (mkdir(sdir.c_str(), 0755) != 0 && errno != EEXIST)
            return report_status(ISLBM_ERR_INVALID_ARGUMENT, ("cannot create " + sdir).c_str());
        return islbm_stats_write(h, sdir.c_str(), rank);
    }
    return ISLBM_OK;
}

// statistics of a checkpoint, when it has them
static int read_stats_if_present(islbm_handle *h, const char *dir, int rank) {
    const std::string sdir = std::string(dir) + "/statistics";
    FILE *fp = std::fopen((sdir + "/accu.dat").c_str(), "r");
    if (!fp) return ISLBM_OK;
    std::fclose(fp);
    return islbm_stats_read(h, sdir.c_str(), rank);
}

int islbm_checkpoint_read(islbm_handle *h, const char *dir, int rank) {
    if (!h || !dir) return ISLBM_ERR_INVALID_ARGUMENT;
    const size_t nref = (size_t)(h->p.NX + 7)*(h->p.NY + 7)*(h->p.NZ + 6);
    std::vector<double> f19(19*nref);
    for (int q = 0; q < 19; q++) {
        const int st = read_raw(path_of(dir, "f" + std::to_string(q), rank), f19.data() + (size_t)q*nref, nref);
        if (st != ISLBM_OK) return st;
    }
    int st = islbm_set_populations(h, f19.data(), ISLBM_LAYOUT_REFERENCE);
    if (st != ISLBM_OK) return st;
    // the macroscopic fields of the file, so that islbm_fields reports them before the next step
    std::vector<double> mref(nref), uni(h->N);
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return report_cuda(e, "cudaSetDevice");
    for (int m = 0; m < 4; m++) {
        st = read_raw(path_of(dir, kMacroNames[m], rank), mref.data(), nref);
        if (st != ISLBM_OK) return st;
        reference_to_unique_layout(h, mref.data(), uni.data());
        if (h->celem == 8) {
            e = cudaMemcpyAsync(h->macros[m], uni.data(), h->N*8, cudaMemcpyHostToDevice, h->stream);
        } else {
            std::vector<float> fl(h->N);
            for (size_t i = 0; i < h->N; i++) fl[i] = (float)uni[i];
            e = cudaMemcpyAsync(h->macros[m], fl.data(), h->N*4, cudaMemcpyHostToDevice, h->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);   // fl goes out of scope
        }
        if (e != cudaSuccess) return report_cuda(e, "checkpoint fields upload");
    }
    e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return report_cuda(e, "checkpoint fields upload");
    // controller: this library's exact record when present, else the reference's force file
    const std::string cpath = std::string(dir) + "/islbm_ctrl_" + std::to_string(rank) + ".bin";
    FILE *fp = std::fopen(cpath.c_str(), "rb");
    if (fp) {
        CtrlFile cf{};
        const size_t r = std::fread(&cf, sizeof(cf), 1, fp);
        std::fclose(fp);
        if (r != 1 || std::memcmp(cf.magic, "ISLBMCK1", 8) != 0)
            return report_status(ISLBM_ERR_INVALID_ARGUMENT, ("bad controller record " + cpath).c_str());
        cf.ctrl.done = 0u;
        cf.ctrl.fault = 0u;
        e = cudaMemcpyAsync(h->ctrl, &cf.ctrl, sizeof(Ctrl), cudaMemcpyHostToDevice, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) return report_cuda(e, "checkpoint controller upload");
        h->steps = cf.steps;
        // keep the buffer of the current state at index (steps mod 2), as stepping leaves it
        if ((int)(h->steps & 1ULL) != h->cur) {
            std::swap(h->fbuf[0], h->fbuf[1]);
            h->cur = (int)(h->steps & 1ULL);
        }
        return read_stats_if_present(h, dir, rank);
    }
    const std::string fpath = std::string(dir) + "/0_force.dat";
    fp = std::fopen(fpath.c_str(), "r");
    if (!fp) return report_status(ISLBM_ERR_INVALID_ARGUMENT, ("cannot read " + fpath).c_str());
    double force = 0.0;
    const int got = std::fscanf(fp, "%lf", &force);
    std::fclose(fp);
    if (got != 1) return report_status(ISLBM_ERR_INVALID_ARGUMENT, ("bad force file " + fpath).c_str());
    st = islbm_set_force(h, force);
    return st != ISLBM_OK ? st : read_stats_if_present(h, dir, rank);
}

}  // extern "C"
