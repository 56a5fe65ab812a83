// Serving loop: continuous batching of many periodic-hill solves on one GPU.
//
// Requests arrive through islbm_server_submit at any time. Each pump:
//   1. admits queued requests in arrival order while the device budget allows (every solve
//      keeps its populations, weight tables and controller resident on the GPU);
//   2. advances every active solve by one chunk of steps: solves that share a storage
//      format and spanwise width are stepped by one batched tiled launch per step, the chunk
//      of launches captured once per batch composition in a CUDA graph and replayed; other
//      solves use their own step kernel;
//   3. measures the relative change of the velocity field of each solve that has completed
//      steps_per_chunk steps since its previous check (one scalar per solve read back) and
//      retires solves that converged, diverged or reached their step cap, freeing their memory
//      for the queue. A chunk ends at the next check or cap of any active solve, so every
//      check of every solve spans exactly steps_per_chunk of its steps, whenever it arrived.
// The launch shape of each batch (persistent CTAs per SM) is picked by a small autotuner that
// times the candidates on the first steps of a new batch composition and caches the winner.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "../../include/islbm_serve.h"
#include "handle.hpp"

namespace islbm {
namespace {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// sum over nodes of |u - u_snap|^2 (FP64 accumulation), then snap <- u
template <class T>
__global__ void delta_kernel(const T *__restrict__ u, const T *__restrict__ v, const T *__restrict__ w,
                             T *__restrict__ snap, size_t n, double *out) {
    double acc = 0.0;
    for (size_t i = blockIdx.x*(size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x*blockDim.x) {
        const double du = (double)u[i] - (double)snap[i], dv = (double)v[i] - (double)snap[n + i],
                     dw = (double)w[i] - (double)snap[2*n + i];
        acc += du*du + dv*dv + dw*dw;
        snap[i] = u[i]; snap[n + i] = v[i]; snap[2*n + i] = w[i];
    }
    __shared__ double red[32];
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += red[i];
        atomicAdd(out, s);
    }
}

template <class T>
__global__ void snap_kernel(const T *u, const T *v, const T *w, T *snap, size_t n) {
    for (size_t i = blockIdx.x*(size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x*blockDim.x) {
        snap[i] = u[i]; snap[n + i] = v[i]; snap[2*n + i] = w[i];
    }
}

// velocity snapshot kernels for a solve's compute type (FP64 solves keep FP64 macros)
cudaError_t launch_snap(const islbm_handle *h, void *snap, cudaStream_t st) {
    const unsigned g = (unsigned)std::min<size_t>(1024, (h->N + 255)/256);
    if (h->celem == 8)
        snap_kernel<double><<<g, 256, 0, st>>>((const double *)h->macros[1], (const double *)h->macros[2],
                                               (const double *)h->macros[3], (double *)snap, h->N);
    else
        snap_kernel<float><<<g, 256, 0, st>>>((const float *)h->macros[1], (const float *)h->macros[2],
                                              (const float *)h->macros[3], (float *)snap, h->N);
    return cudaGetLastError();
}

cudaError_t launch_delta(const islbm_handle *h, void *snap, double *out, cudaStream_t st) {
    const unsigned g = (unsigned)std::min<size_t>(1024, (h->N + 255)/256);
    if (h->celem == 8)
        delta_kernel<double><<<g, 256, 0, st>>>((const double *)h->macros[1], (const double *)h->macros[2],
                                                (const double *)h->macros[3], (double *)snap, h->N, out);
    else
        delta_kernel<float><<<g, 256, 0, st>>>((const float *)h->macros[1], (const float *)h->macros[2],
                                               (const float *)h->macros[3], (float *)snap, h->N, out);
    return cudaGetLastError();
}

struct Solve {
    long long id = 0;
    islbm_params p{};
    long long max_steps = 0;
    double tol = 0.0;
    int keep = 0;
    islbm_handle *h = nullptr;
    void *snap = nullptr;       // velocity at the previous convergence check (compute type)
    size_t bytes = 0;
    long long steps = 0;
    long long since_check = 0;  // steps since the previous convergence check (or admission)
    double delta = -1.0;
    int status = ISLBM_SOLVE_QUEUED;
    double t_submit = 0, t_admit = 0, t_done = 0;
    double force = 0.0;
    std::vector<double> fields;   // rho, u, v, w (unique layout) kept after retirement
};

struct Group {
    int precision = 0, NX = 0;
    bool les = false;
    bool paired = false;         // members step with the paired-node kernel (step_pair.cu)
    std::vector<Solve *> members;
    void *descs = nullptr;       // device descriptors
    int2 *items = nullptr;       // device (solve, segment*ntiles + tile) work list
    int nitems = 0;
    long long nodes = 0;         // lattice nodes updated per step
    int grid = 0;
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0;
    std::string key;
    cudaStream_t stream = nullptr;   // batches run side by side, each on its own stream
    cudaEvent_t done = nullptr;      // end of this batch's chunk
};

}  // namespace
}  // namespace islbm

using namespace islbm;

struct islbm_server {
    int device = 0;
    cudaStream_t stream = nullptr;
    size_t budget = 0, used = 0;
    int chunk = 500;
    int sms = 0;
    long long next_id = 1;
    double t0 = 0;
    std::deque<Solve *> queue;
    std::vector<Solve *> active;
    std::map<long long, std::unique_ptr<Solve>> all;
    std::map<std::string, std::unique_ptr<Group>> groups;
    std::map<std::string, int> tuned_grid;   // autotuner cache: batch signature -> CTAs
    double *dsum = nullptr;                  // per-solve delta sums (device)
    size_t dsum_cap = 0;
    long long updates = 0;                   // lattice-node updates performed
    double busy = 0.0;                       // seconds inside pump
    std::string last;
};

namespace {

int fail(islbm_server *s, cudaError_t e, const char *what) {
    s->last = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? ISLBM_ERR_OUT_OF_MEMORY : ISLBM_ERR_CUDA;
}
#define SK(call)                                             \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return fail(s, e_, #call);    \
    } while (0)

size_t solve_bytes(const islbm_params &p) {
    size_t b = 0;
    islbm_required_bytes(&p, &b);
    const size_t ce = p.precision == ISLBM_FP64 ? 8 : 4;
    return b + 3*(size_t)p.NX*p.NY*p.NZ*ce;
}

void free_group(Group *g) {
    if (g->stream) cudaStreamSynchronize(g->stream);
    if (g->graph) cudaGraphExecDestroy(g->graph);
    if (g->descs) cudaFree(g->descs);
    if (g->items) cudaFree(g->items);
    if (g->done) cudaEventDestroy(g->done);
    if (g->stream) cudaStreamDestroy(g->stream);
    g->graph = nullptr; g->descs = nullptr; g->items = nullptr; g->done = nullptr; g->stream = nullptr;
}

// batched launches advance a solve on the device (its controller's step counter picks the
// buffers); keep the handle's host view in step so that islbm_fields and friends read the
// current buffer
void advanced(islbm_server *s, Group *g, int steps) {
    for (Solve *v : g->members) {
        v->steps += steps;
        v->h->steps += (unsigned long long)steps;
        v->h->cur = (int)(v->h->steps & 1ULL);
    }
    s->updates += (long long)steps*g->nodes;
}

void retire(islbm_server *s, Solve *v, int status) {
    v->status = status;
    v->t_done = now_s() - s->t0;
    if (v->keep) {
        const size_t n = (size_t)v->p.NX*v->p.NY*v->p.NZ;
        v->fields.assign(4*n, 0.0);
        islbm_fields(v->h, v->fields.data(), v->fields.data() + n, v->fields.data() + 2*n, v->fields.data() + 3*n,
                     ISLBM_LAYOUT_UNIQUE);
    }
    double f = 0;
    islbm_get_scalars(v->h, &f, nullptr, nullptr);
    v->force = f;
    if (v->snap) cudaFree(v->snap);
    v->snap = nullptr;
    handle_free(v->h);
    v->h = nullptr;
    s->used -= v->bytes;
}

// Admit queued requests in arrival order while the budget allows; the new solves are appended
// to `fresh` (they join the active set when the caller says so).
int admit(islbm_server *s, std::vector<Solve *> &fresh) {
    while (!s->queue.empty()) {
        Solve *v = s->queue.front();
        if (s->used + v->bytes > s->budget && !(s->active.empty() && fresh.empty())) break;   // wait for memory
        if (s->used + v->bytes > s->budget) {   // can never fit
            s->queue.pop_front();
            v->status = ISLBM_SOLVE_REJECTED;
            v->t_done = now_s() - s->t0;
            continue;
        }
        s->queue.pop_front();
        islbm_params p = v->p;
        p.device = s->device;
        p.kernel = ISLBM_KERNEL_AUTO;
        islbm_handle *h = new (std::nothrow) islbm_handle();
        if (!h) return ISLBM_ERR_OUT_OF_MEMORY;
        int st = handle_init(&p, h);
        if (st != ISLBM_OK) { handle_free(h); v->status = ISLBM_SOLVE_REJECTED; v->t_done = now_s() - s->t0; continue; }
        v->h = h;
        const size_t n = h->N;
        SK(cudaMalloc(&v->snap, 3*n*h->celem));
        // the macro buffers hold the initial state's velocity after islbm_init
        SK(launch_snap(h, v->snap, s->stream));
        v->status = ISLBM_SOLVE_ACTIVE;
        v->t_admit = now_s() - s->t0;
        s->used += v->bytes;
        fresh.push_back(v);
    }
    return ISLBM_OK;
}

// Build (or reuse) the batch groups for the current active set.
int build_groups(islbm_server *s, std::vector<Group *> &out, std::vector<Solve *> &singles) {
    std::map<std::string, std::vector<Solve *>> by;
    for (Solve *v : s->active) {
        islbm_handle *h = v->h;
        if (!h->use_tiled) { singles.push_back(v); continue; }
        const std::string sig = std::to_string(h->p.precision) + "/" + std::to_string(h->p.NX) + "/" +
                                std::to_string(h->p.les_cs > 0.0 ? 1 : 0) + "/" + std::to_string(h->paired ? 1 : 0);
        by[sig].push_back(v);
    }
    for (auto &kv : by) {
        std::string key = kv.first + ":";
        for (Solve *v : kv.second) key += std::to_string(v->id) + ",";
        auto it = s->groups.find(kv.first);
        if (it != s->groups.end() && it->second->key == key) { out.push_back(it->second.get()); continue; }
        if (it != s->groups.end()) { free_group(it->second.get()); s->groups.erase(it); }
        auto g = std::make_unique<Group>();
        islbm_handle *h0 = kv.second[0]->h;
        g->precision = h0->p.precision; g->NX = h0->p.NX; g->les = h0->p.les_cs > 0.0; g->paired = h0->paired;
        g->members = kv.second;
        g->key = key;
        const size_t db = g->paired ? pair_batch_desc_bytes(g->precision, g->NX, g->les)
                                    : batch_desc_bytes(g->precision, g->NX, g->les);
        std::vector<unsigned char> hd(db*g->members.size());
        std::vector<int2> items;
        int maxt = 0, total_tiles = 0, min_nz = 1 << 30;
        for (size_t m = 0; m < g->members.size(); m++) {
            islbm_handle *h = g->members[m]->h;
            const int ntiles = h->p.NY/h->tiled.TY;
            maxt = std::max(maxt, ntiles);
            total_tiles += ntiles;
            min_nz = std::min(min_nz, h->p.NZ);
        }
        // wall-normal segments per column: enough work items for four CTAs per SM, each segment
        // at least 16 targets long (a segment re-reads the 6 planes below it to fill its ring)
        // (paired kernel: two CTAs per SM, segment count by the makespan estimate of pair_zsegs)
        const int nseg = g->paired ? pair_zsegs(total_tiles, 2*s->sms, min_nz)
                                   : std::max(1, std::min(4*s->sms/std::max(1, total_tiles), min_nz/16));
        for (size_t m = 0; m < g->members.size(); m++) {
            islbm_handle *h = g->members[m]->h;
            g->nodes += (long long)h->N;
            (g->paired ? fill_pair_batch_desc : fill_batch_desc)(g->precision, g->NX, g->les, h->tf, h->k, h->tiled, h->ctrl, h->macros, h->fbuf[0], h->fbuf[1],
                            h->p.NY/h->tiled.TY, nseg, hd.data() + m*db);
        }
        // segment-major, the solves' tiles interleaved, so that neighbouring tiles of a solve at
        // the same height run together
        for (int seg = 0; seg < nseg; seg++)
            for (int t = 0; t < maxt; t++)
                for (size_t m = 0; m < g->members.size(); m++) {
                    islbm_handle *h = g->members[m]->h;
                    const int nt = h->p.NY/h->tiled.TY;
                    if (t < nt) items.push_back(make_int2((int)m, seg*nt + t));
                }
        g->nitems = (int)items.size();
        SK(cudaMalloc(&g->descs, hd.size()));
        SK(cudaMalloc(&g->items, items.size()*sizeof(int2)));
        SK(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
        SK(cudaEventCreateWithFlags(&g->done, cudaEventDisableTiming));
        SK(cudaMemcpyAsync(g->descs, hd.data(), hd.size(), cudaMemcpyHostToDevice, g->stream));
        SK(cudaMemcpyAsync(g->items, items.data(), items.size()*sizeof(int2), cudaMemcpyHostToDevice, g->stream));
        out.push_back(g.get());
        s->groups[kv.first] = std::move(g);
    }
    // drop groups that no longer have members
    for (auto it = s->groups.begin(); it != s->groups.end();) {
        bool used = false;
        for (Group *g : out) used |= (g == it->second.get());
        if (!used) { free_group(it->second.get()); it = s->groups.erase(it); } else ++it;
    }
    return ISLBM_OK;
}

// one batched step of every member of g on the group's stream
cudaError_t launch_batch(Group *g, int grid, int macros_on) {
    return g->paired ? launch_step_pair_batch(g->precision, g->NX, g->les, g->descs, g->items, g->nitems, grid, macros_on, g->stream)
                     : launch_step_tiled_batch(g->precision, g->NX, g->les, g->descs, g->items, g->nitems, grid, macros_on, g->stream);
}

// Autotuner: candidate persistent-CTA counts for a batch, timed on one real step each.
// Returns a status; the timed launches advance every member and are accounted for here.
// Picks the group's CTA count. The timed candidate launches are real steps of every member:
// at most `budget` of them, their number returned in `launched`.
int tune(islbm_server *s, Group *g, int budget, int &launched) {
    launched = 0;
    const std::string sig = std::to_string(g->precision) + "/" + std::to_string(g->NX) + "/" + std::to_string(g->les) +
                            "/" + std::to_string(g->nitems);
    auto it = s->tuned_grid.find(sig);
    if (it != s->tuned_grid.end()) { g->grid = it->second; return ISLBM_OK; }
    const int cand[3] = {std::min(g->nitems, s->sms), std::min(g->nitems, 2*s->sms), std::min(g->nitems, 4*s->sms)};
    // the tuning steps must fit in this chunk (they count toward it); otherwise this batch
    // composition keeps the default shape
    if (budget < 3) { g->grid = cand[1]; return ISLBM_OK; }
    float best = 1e30f;
    int best_grid = cand[0];
    cudaEvent_t e0, e1;
    SK(cudaEventCreate(&e0));
    SK(cudaEventCreate(&e1));
    for (int c = 0; c < 3; c++) {
        if (c > 0 && cand[c] == cand[c - 1]) continue;
        SK(cudaEventRecord(e0, g->stream));
        SK(launch_batch(g, cand[c], 1));
        SK(cudaEventRecord(e1, g->stream));
        SK(cudaEventSynchronize(e1));
        launched++;
        float ms = 0;
        SK(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) { best = ms; best_grid = cand[c]; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    advanced(s, g, launched);   // the timed launches are real steps of every member
    s->tuned_grid[sig] = best_grid;
    g->grid = best_grid;
    return ISLBM_OK;
}

int run_group_chunk(islbm_server *s, Group *g, int steps) {
    if (!g->graph || g->graph_steps != steps) {
        if (g->graph) cudaGraphExecDestroy(g->graph);
        g->graph = nullptr;
        cudaGraph_t graph;
        SK(g->paired ? prepare_step_pair_batch(g->precision, g->NX, g->les) : prepare_step_tiled_batch(g->precision, g->NX, g->les));
        SK(cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal));
        for (int j = 0; j < steps; j++) {
            cudaError_t e = launch_batch(g, g->grid, j == steps - 1);
            if (e != cudaSuccess) { cudaStreamEndCapture(g->stream, &graph); return fail(s, e, "batched step capture"); }
        }
        SK(cudaStreamEndCapture(g->stream, &graph));
        SK(cudaGraphInstantiate(&g->graph, graph, 0));
        cudaGraphDestroy(graph);
        g->graph_steps = steps;
    }
    SK(cudaGraphLaunch(g->graph, g->stream));
    return ISLBM_OK;
}

}  // namespace

extern "C" {

int islbm_server_create(int device, size_t hbm_budget_bytes, int steps_per_chunk, islbm_server **out) {
    if (!out || steps_per_chunk < 1) return ISLBM_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return ISLBM_ERR_NO_DEVICE;
    if (device < 0 || device >= ndev) return ISLBM_ERR_INVALID_ARGUMENT;
    islbm_server *s = new (std::nothrow) islbm_server();
    if (!s) return ISLBM_ERR_OUT_OF_MEMORY;
    s->device = device;
    s->budget = hbm_budget_bytes ? hbm_budget_bytes : (size_t)150 << 30;
    s->chunk = steps_per_chunk;
    s->t0 = now_s();
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
        delete s;
        return ISLBM_ERR_CUDA;
    }
    *out = s;
    return ISLBM_OK;
}

int islbm_server_submit(islbm_server *s, const islbm_params *p, long long max_steps, double tol, int keep_fields,
                        long long *id) {
    if (!s || !p || max_steps < 1 || !(tol >= 0.0)) return ISLBM_ERR_INVALID_ARGUMENT;
    const int st = validate(*p);
    if (st != ISLBM_OK) return st;
    auto v = std::make_unique<Solve>();
    v->id = s->next_id++;
    v->p = *p;
    v->max_steps = max_steps;
    v->tol = tol;
    v->keep = keep_fields;
    v->bytes = solve_bytes(*p);
    v->t_submit = now_s() - s->t0;
    s->queue.push_back(v.get());
    if (id) *id = v->id;
    s->all[v->id] = std::move(v);
    return ISLBM_OK;
}

int islbm_server_pump(islbm_server *s, int *n_active, int *n_queued) {
    if (!s) return ISLBM_ERR_INVALID_ARGUMENT;
    const double t_start = now_s();
    SK(cudaSetDevice(s->device));
    std::vector<Solve *> fresh;
    int st = ISLBM_OK;
    if (s->active.empty()) {   // nothing on the device: admit now
        st = admit(s, fresh);
        if (st != ISLBM_OK) return st;
        s->active.swap(fresh);
        fresh.clear();
    }
    if (!s->active.empty()) {
        // chunk length: up to the next convergence check or step cap of any active solve
        int steps = s->chunk;
        for (Solve *v : s->active)
            steps = (int)std::min<long long>(steps, std::max<long long>(1, std::min<long long>(s->chunk - v->since_check,
                                                                                             v->max_steps - v->steps)));
        std::vector<Group *> groups;
        std::vector<Solve *> singles;
        st = build_groups(s, groups, singles);
        if (st != ISLBM_OK) return st;
        for (Group *g : groups) {
            int tuned = 0;
            if (!g->grid) {
                st = tune(s, g, steps, tuned);
                if (st != ISLBM_OK) return st;
            }
            // the tuning steps count toward the chunk; what remains runs as one graph
            const int left = steps - tuned;
            if (left > 0) {
                st = run_group_chunk(s, g, left);
                if (st != ISLBM_OK) return st;
                advanced(s, g, left);
            }
        }
        for (Solve *v : singles) {
            // solves without a batched layout: their own kernel on their own stream
            st = islbm_step(v->h, steps);
            if (st != ISLBM_OK) return st;
            v->steps += steps;
            s->updates += (long long)steps*(long long)v->h->N;
        }
        for (Solve *v : s->active) v->since_check += steps;
        // the convergence measure (on the server stream) waits for every batch
        for (Group *g : groups) {
            SK(cudaEventRecord(g->done, g->stream));
            SK(cudaStreamWaitEvent(s->stream, g->done, 0));
        }
        // while the chunk runs: set up the requests that arrived (host precompute, uploads on
        // their own streams); they join the active set after this chunk
        st = admit(s, fresh);
        if (st != ISLBM_OK) return st;
        for (Solve *v : singles) {
            st = islbm_sync(v->h);
            if (st != ISLBM_OK) return st;
        }
        // convergence measure of every active solve
        if (s->dsum_cap < s->active.size()) {
            if (s->dsum) cudaFree(s->dsum);
            s->dsum_cap = s->active.size() + 16;
            SK(cudaMalloc(&s->dsum, s->dsum_cap*sizeof(double)));
        }
        SK(cudaMemsetAsync(s->dsum, 0, s->active.size()*sizeof(double), s->stream));
        // only solves at the end of a full check interval are measured (their snapshot advances)
        for (size_t i = 0; i < s->active.size(); i++)
            if (s->active[i]->since_check >= s->chunk) SK(launch_delta(s->active[i]->h, s->active[i]->snap, s->dsum + i, s->stream));
        std::vector<double> sums(s->active.size());
        SK(cudaMemcpyAsync(sums.data(), s->dsum, sums.size()*sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        SK(cudaStreamSynchronize(s->stream));
        std::vector<Solve *> keep;
        for (size_t i = 0; i < s->active.size(); i++) {
            Solve *v = s->active[i];
            const double n = (double)v->h->N;
            const bool checked = v->since_check >= s->chunk;
            if (checked) {
                v->delta = std::sqrt(sums[i]/n)/v->p.Uref;
                v->since_check = 0;
            }
            // a timed-out pipeline wait in the step kernel leaves the state undefined
            st = islbm_sync(v->h);
            if (st != ISLBM_OK) { s->last = "step kernel pipeline wait timed out"; return st; }
            long long bad = 0;
            const int fin = islbm_check_finite(v->h, &bad);
            // a change of the velocity by more than a thousand times the bulk velocity between two
            // checks only happens on the way to overflow
            if (fin != ISLBM_OK || !(v->delta <= 1e3)) retire(s, v, ISLBM_SOLVE_DIVERGED);
            else if (checked && v->delta < v->tol) retire(s, v, ISLBM_SOLVE_CONVERGED);
            else if (v->steps >= v->max_steps) retire(s, v, ISLBM_SOLVE_CAPPED);
            else keep.push_back(v);
        }
        s->active.swap(keep);
        for (Solve *v : fresh) s->active.push_back(v);
    }
    s->busy += now_s() - t_start;
    if (n_active) *n_active = (int)s->active.size();
    if (n_queued) *n_queued = (int)s->queue.size();
    return ISLBM_OK;
}

int islbm_server_info(islbm_server *s, long long id, islbm_solve_info *out) {
    if (!s || !out) return ISLBM_ERR_INVALID_ARGUMENT;
    auto it = s->all.find(id);
    if (it == s->all.end()) return ISLBM_ERR_INVALID_ARGUMENT;
    const Solve *v = it->second.get();
    out->id = v->id;
    out->status = v->status;
    out->steps = v->steps;
    out->delta = v->delta;
    out->t_submit = v->t_submit;
    out->t_admit = v->t_admit;
    out->t_done = v->t_done;
    out->force = v->force;
    out->nodes = (long long)v->p.NX*v->p.NY*v->p.NZ;
    return ISLBM_OK;
}

int islbm_server_fields(islbm_server *s, long long id, double *rho, double *u, double *v, double *w) {
    if (!s) return ISLBM_ERR_INVALID_ARGUMENT;
    auto it = s->all.find(id);
    if (it == s->all.end()) return ISLBM_ERR_INVALID_ARGUMENT;
    Solve *x = it->second.get();
    if (x->h) return islbm_fields(x->h, rho, u, v, w, ISLBM_LAYOUT_UNIQUE);
    if (x->fields.empty()) return ISLBM_ERR_NOT_SUPPORTED;
    const size_t n = x->fields.size()/4;
    double *dst[4] = {rho, u, v, w};
    for (int m = 0; m < 4; m++)
        if (dst[m]) std::memcpy(dst[m], x->fields.data() + m*n, n*sizeof(double));
    return ISLBM_OK;
}

int islbm_server_stats(islbm_server *s, long long *updates, double *busy_seconds, size_t *bytes_in_use) {
    if (!s) return ISLBM_ERR_INVALID_ARGUMENT;
    if (updates) *updates = s->updates;
    if (busy_seconds) *busy_seconds = s->busy;
    if (bytes_in_use) *bytes_in_use = s->used;
    return ISLBM_OK;
}

int islbm_server_destroy(islbm_server *s) {
    if (!s) return ISLBM_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->device);
    for (auto &kv : s->groups) free_group(kv.second.get());
    for (Solve *v : s->active) {
        if (v->snap) cudaFree(v->snap);
        handle_free(v->h);
    }
    if (s->dsum) cudaFree(s->dsum);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return ISLBM_OK;
}

}  // extern "C"
