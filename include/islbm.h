/* islbm.h - C ABI of the GB300 ISLBM periodic-hill step library (libislbm_gb300.so).
 *
 * Drop-in for the reference solver's step path (ChenPengChung/Lattie-Boltzmann-Method-Note_of_
 * PaperReView, directory 筆記：金的code/0.可更改的code/, cited below as C/):
 *   islbm_init    replaces AllocateMemory + GenerateMesh_X/Y/Z + GetIntrplParameter_X/Y/Xi +
 *                 BFLInitialization + InitialUsingDftFunc + SendDataToGPU
 *                 (C/memory.h:51, C/initialization.h:6-360, C/communication.h:245)
 *   islbm_step    replaces n calls of Launch_CollisionStreaming(f_old, f_new) with the
 *                 ft/fd ping-pong of the main loop, AccumulateUbulk, and
 *                 Launch_ModifyForcingTerm every NDTFRC steps (C/evolution.h:826-1042)
 *   islbm_fields  replaces SendDataToCPU for rho, u, v, w (C/communication.h:260-273)
 *   islbm_destroy replaces FreeSource (C/memory.h:173)
 * The whole domain lives on one GPU; the reference's MPI halo exchange and periodic ghost
 * kernels are replaced by in-kernel periodic wrap.
 *
 * Axes and names follow the reference (C/variables.h): x = spanwise (NX, LX, periodic),
 * y = streamwise (NY, LY, periodic, hill and body force along y), z = wall-normal (NZ, LZ,
 * body-fitted). u, v, w are the x, y, z velocity components.
 *
 * Conventions: every function returns an islbm_status; no function calls exit(). Host
 * buffers belong to the caller, device buffers to the handle. A handle owns one CUDA stream;
 * use one handle per host thread (calls on one handle are not thread-safe).
 */
#ifndef ISLBM_H
#define ISLBM_H

#include <stddef.h>

#if defined(__GNUC__)
#define ISLBM_API __attribute__((visibility("default")))
#else
#define ISLBM_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum islbm_status {
    ISLBM_OK = 0,
    ISLBM_ERR_INVALID_ARGUMENT = 1,
    ISLBM_ERR_CUDA = 2,
    ISLBM_ERR_OUT_OF_MEMORY = 3,
    ISLBM_ERR_HBM_BUDGET = 4,      /* the solve does not fit the handle's HBM budget */
    ISLBM_ERR_NONFINITE = 5,       /* a NaN/Inf was found in the state */
    ISLBM_ERR_NOT_SUPPORTED = 6,
    ISLBM_ERR_NO_DEVICE = 7
} islbm_status;

typedef enum islbm_precision {
    ISLBM_FP64 = 0,       /* distributions and arithmetic in FP64 (parity path) */
    ISLBM_FP32 = 1,       /* distributions and arithmetic in FP32 */
    ISLBM_FP16_DEV = 2,   /* distributions stored as FP16 deviations f_i - feq_i(rho 1, u = 0.05 e_y), FP32 arithmetic */
    ISLBM_BF16_DEV = 3    /* distributions stored as BF16 deviations, as FP16_DEV, FP32 arithmetic */
} islbm_precision;

typedef enum islbm_layout {
    ISLBM_LAYOUT_UNIQUE = 0,     /* NZ x NY x NX unique nodes, x fastest: [z][y][x] */
    ISLBM_LAYOUT_REFERENCE = 1   /* NYD6 x NZ6 x NX6 with ghosts, index j*NX6*NZ6 + k*NX6 + i
                                    (C/initialization.h:20); periodic ghosts and the duplicated
                                    end nodes are filled, the z ghost layers are zero */
} islbm_layout;

typedef enum islbm_kernel {
    ISLBM_KERNEL_AUTO = 0,       /* tiled kernel when the grid allows it, else gather kernel */
    ISLBM_KERNEL_GATHER = 1,     /* one thread per node, stencils read through L1/L2 */
    ISLBM_KERNEL_TILED = 2,      /* z-marching x-y tiles staged in shared memory (two nodes per
                                    thread where the width allows it, else one) */
    ISLBM_KERNEL_TILED_SINGLE = 3 /* the tiled kernel with one node per thread */
} islbm_kernel;

/* Parameter set of C/variables.h (same names where the reference has one). */
typedef struct islbm_params {
    int NX, NY, NZ;            /* grid: spanwise, streamwise, wall-normal */
    double LX, LY, LZ;         /* domain (4.5, 9.0, 3.036; hill height 1) */
    double CFL;                /* minSize = (LZ-1)/NZ*CFL, dt = minSize */
    double LXi;                /* computational extent of the xi coordinate (10.0) */
    double Re;                 /* Reynolds number on hill height and Uref */
    double Uref;               /* bulk velocity; tau = 0.5 + 3*Uref/(Re*minSize) */
    int NDTFRC;                /* forcing-controller period in steps (C/variables.h:48) */
    int precision;             /* islbm_precision */
    double les_cs;             /* Smagorinsky constant (0 = plain MRT) */
    double alpha;              /* hill steepness: footprint scaled by alpha (1 = reference) */
    int init_mode;             /* 0: rest state of InitialUsingDftFunc; 1: v = Uref + noise */
    unsigned long long seed;   /* noise seed for init_mode 1 */
    double perturb;            /* noise amplitude relative to Uref (0.01 = +/-1 %) */
    int mass_interval;         /* rho_modify every mass_interval steps (0 = off) */
    int bfl_mode;              /* 0: BFL weight tables indexed as the reference does (x by i,
                                  y by j, C/evolution.h:525-527); 1: by the wall row */
    int device;                /* CUDA device ordinal */
    int kernel;                /* islbm_kernel */
    size_t hbm_budget_bytes;   /* refuse solves above this many device bytes (0 = no limit) */
    int geometry;              /* 0: periodic hill (HillFunction, C/model.h:4-68); 1: flat channel
                                  (ChannelFunction, C/model.h:70-73) */
} islbm_params;

typedef struct islbm_handle islbm_handle;

/* Fill `p` with the reference's defaults (C/variables.h) and the 64x32x48 hill case. */
ISLBM_API int islbm_default_params(islbm_params *p);

/* Device bytes islbm_init would allocate for `p` (no device needed). */
ISLBM_API int islbm_required_bytes(const islbm_params *p, size_t *bytes);

/* Build mesh, weights and BFL tables in FP64 on the host, upload them, set the initial
 * state and the initial body force (C/initialization.h:46). */
ISLBM_API int islbm_init(const islbm_params *p, islbm_handle **out);

/* Advance nsteps lattice steps (asynchronous on the handle's stream). The macroscopic
 * fields of the last step are kept for islbm_fields. */
ISLBM_API int islbm_step(islbm_handle *h, int nsteps);

/* Copy rho, u, v, w of the last step to host buffers (FP64, `layout`); any pointer may be
 * NULL. Before the first step these are the initial fields. Synchronises the stream. */
ISLBM_API int islbm_fields(islbm_handle *h, double *rho, double *u, double *v, double *w, int layout);

/* Copy population q (full value f_q, FP64) of the current state to a host buffer. */
ISLBM_API int islbm_get_population(islbm_handle *h, int q, double *out, int layout);

/* Replace the current state: f19 holds 19 consecutive arrays in `layout` (FP64). Restart
 * path of InitialUsingBkpData (C/fileIO.h:315-354). */
ISLBM_API int islbm_set_populations(islbm_handle *h, const double *f19, int layout);

/* Controller state: body force (Force_d), mass correction (rho_modify_d), steps taken. */
ISLBM_API int islbm_get_scalars(islbm_handle *h, double *force, double *rho_modify, long long *steps);
ISLBM_API int islbm_set_force(islbm_handle *h, double force);

/* Derived constants: tau, niu, Uref, minSize (C/variables.h:22, 76, 97-101). */
ISLBM_API int islbm_get_constants(islbm_handle *h, double *tau, double *niu, double *uref, double *min_size);

/* Device bytes of the weight tables as stored (per (y, z, direction)) and as they would be
 * stored per node. */
ISLBM_API int islbm_weight_table_bytes(islbm_handle *h, size_t *stored, size_t *per_node);

/* The handle's CUDA stream (cudaStream_t) for event timing by the caller. */
ISLBM_API int islbm_get_stream(islbm_handle *h, void **stream);

/* Wait for all work on the handle's stream; returns ISLBM_ERR_CUDA on a device error. */
ISLBM_API int islbm_sync(islbm_handle *h);

/* Count non-finite values in the current state (0 = healthy). */
ISLBM_API int islbm_check_finite(islbm_handle *h, long long *bad);

/* Whole-field diagnostics from the current populations (FP64 reduction over unique nodes):
 * out[0] total mass sum(rho), out[1] mean streamwise momentum sum(rho v)/N, out[2] kinetic
 * energy sum(rho |u|^2)/2, out[3] maximum speed max|u|. Replaces the host-side mass check of
 * the reference main loop (all populations copied by SendDataToCPU, C/communication.h:260-273,
 * every 100 steps) and extends the Monitor.dat record (C/monitor.h:4-26). Allocates a scratch
 * buffer of 512 + 32*ceil(N/2048) bytes on the device for the call and frees it. */
ISLBM_API int islbm_diagnostics(islbm_handle *h, double *out);
/* The same diagnostics without any device allocation. No reference counterpart: the reference
 * has no such call. It is for callers that cannot allocate device memory during a run: a
 * serving loop whose device budget is committed to the byte, or code that must not call
 * cudaFree (it waits for all work on the device). Instead of a per-call buffer it uses one
 * fixed scratch array of 524,800 bytes in device memory (per device), so it serves grids of
 * at most 33,554,432 nodes (NX*NY*NZ); larger grids get ISLBM_ERR_NOT_SUPPORTED with a message,
 * and islbm_diagnostics serves them. The first call on a device looks up the scratch address
 * on that device (cudaGetSymbolAddress): make that first call before any stream capture.
 * Calls that overlap in time (other threads, or other handles on the same device) share the
 * scratch and race: run them one at a time. */
ISLBM_API int islbm_diagnostics_noalloc(islbm_handle *h, double *out);

/* Time-averaged statistics (MeanVars of C/statistics.h:122-174, enabled there by TBSWITCH,
 * C/variables.h:32): per-node FP64 sums of the quantities below over samples of the current
 * macroscopic fields, with P = rho/3 - 1/3 and KT = (u^2 + v^2 + w^2)/2. Call
 * islbm_stats_accumulate after islbm_step (which leaves the fields of its last step); the first
 * call allocates ISLBM_STAT_COUNT*N doubles on the device. The reference's velocity-gradient
 * statistics (MeanDerivatives, C/statistics.h:176-222) are not provided: their wall-normal
 * weights (ZSlopePara) are never set in the reference. */
typedef enum islbm_stat {
    ISLBM_STAT_U = 0, ISLBM_STAT_V, ISLBM_STAT_W, ISLBM_STAT_P,
    ISLBM_STAT_UU, ISLBM_STAT_UV, ISLBM_STAT_UW, ISLBM_STAT_VV, ISLBM_STAT_VW, ISLBM_STAT_WW,
    ISLBM_STAT_PU, ISLBM_STAT_PV, ISLBM_STAT_PW, ISLBM_STAT_PP, ISLBM_STAT_KT,
    ISLBM_STAT_UUU, ISLBM_STAT_UUV, ISLBM_STAT_UUW, ISLBM_STAT_VVU, ISLBM_STAT_VVV, ISLBM_STAT_VVW,
    ISLBM_STAT_WWU, ISLBM_STAT_WWV, ISLBM_STAT_WWW,
    ISLBM_STAT_COUNT,
    /* squared velocity gradients (MeanDerivatives, C/statistics.h:176-222), accumulated when
     * enabled with islbm_stats_gradients */
    ISLBM_STAT_DUDX2 = ISLBM_STAT_COUNT, ISLBM_STAT_DUDY2, ISLBM_STAT_DUDZ2,
    ISLBM_STAT_DVDX2, ISLBM_STAT_DVDY2, ISLBM_STAT_DVDZ2,
    ISLBM_STAT_DWDX2, ISLBM_STAT_DWDY2, ISLBM_STAT_DWDZ2,
    ISLBM_STAT_ALL
} islbm_stat;
/* zero the sums (allocating them on first use) */
ISLBM_API int islbm_stats_reset(islbm_handle *h);
/* also accumulate the nine squared velocity gradients (on = 1), from the next reset on: x and y
 * derivatives by the reference's fourth-order central differences, z derivatives by the
 * five-point Lagrange derivative through the column's own wall-normal nodes (the reference
 * indexes its five z weights, ZSlopePara, by k only and never fills them). */
ISLBM_API int islbm_stats_gradients(islbm_handle *h, int on);
/* add one sample (the fields of the last step); asynchronous on the handle's stream */
ISLBM_API int islbm_stats_accumulate(islbm_handle *h);
ISLBM_API int islbm_stats_samples(islbm_handle *h, long long *samples);
/* time mean (sum / samples) of one quantity, unique or reference layout (the reference writes
 * these fields with OutputData, C/fileIO.h:52-67) */
ISLBM_API int islbm_stats_mean(islbm_handle *h, int quantity, double *out, int layout);
/* spanwise average of the time mean at streamwise row y (0 <= y < NY): NZ values, wall-normal
 * index 0 at the hill surface (the profiles of C/fileIO.h:118-249) */
ISLBM_API int islbm_stats_profile(islbm_handle *h, int quantity, int y, double *out);
/* skin friction along the lower wall from the time means: cf[y] = 2 niu (d u_t / d n) / Uref^2
 * for every streamwise row y (NY values), u_t the spanwise-averaged mean velocity tangential to
 * the hill surface, its wall-normal gradient from a quadratic through the wall (half a cell
 * below the first node, where the half-way bounce-back puts it) and the two lowest nodes. */
ISLBM_API int islbm_stats_wall_shear(islbm_handle *h, double *cf);

/* Statistics files of the reference, so that the time means survive a restart (Launch_OutputTB
 * and InitialTBUsingBkpData, C/fileIO.h:356-500): <dir>/accu.dat holds the sample count, and the
 * running sum of each quantity is <dir>/<NAME>/<NAME>_<rank>.bin (NAME = U, V, W, P, UU, ...,
 * WWW, DUDX2, ... as islbm_stat), raw FP64 over k = 3..NZ6-4, j = 3..NYD6-4, i = 3..NX6-4 of the
 * padded layout, k outermost. Write creates the per-quantity directories inside `dir` (which
 * must exist); read replaces the current sums and sample count (gradient quantities are read
 * when islbm_stats_gradients is on). */
ISLBM_API int islbm_stats_write(islbm_handle *h, const char *dir, int rank);
ISLBM_API int islbm_stats_read(islbm_handle *h, const char *dir, int rank);

/* Checkpoint / restart in the reference's files (OutputData / InitialUsingBkpData,
 * C/fileIO.h:52-67, 262-266, 298-354): <dir>/{rho,u,v,w,f0..f18}_<rank>.bin as raw FP64 arrays
 * of NX6*NZ6*NYD6 values in the padded layout, and the body force as text in <dir>/0_force.dat.
 * The controller state (force, bulk-velocity window, step counter) is also written to
 * <dir>/islbm_ctrl_<rank>.bin; read uses it when present (exact resume) and otherwise the text
 * force, as the reference does. The directory must exist. When statistics are being accumulated,
 * write also stores them with islbm_stats_write in <dir>/statistics (created), and read restores
 * them from there when <dir>/statistics/accu.dat exists, so the time means continue exactly. */
ISLBM_API int islbm_checkpoint_write(islbm_handle *h, const char *dir, int rank);
ISLBM_API int islbm_checkpoint_read(islbm_handle *h, const char *dir, int rank);

/* Result files of the reference from the current fields: the Tecplot ASCII velocity file of
 * fileIO_velocity (C/fileIO.h:69-87), the Tecplot binary file of Output3Dvelocity
 * (C/fileIO.h:502-659, velocities / Uref) and one appended Monitor.dat line of Launch_Monitor
 * (C/monitor.h:4-26: step, v, u, w at the centre node, force). */
ISLBM_API int islbm_write_tecplot_ascii(islbm_handle *h, const char *path);
ISLBM_API int islbm_write_tecplot_plt(islbm_handle *h, const char *path);
ISLBM_API int islbm_write_monitor(islbm_handle *h, const char *path, int step);

ISLBM_API int islbm_destroy(islbm_handle *h);

ISLBM_API const char *islbm_status_string(int status);

/* Host-side precompute tables for a parameter set, no device needed (reference layout
 * indexing, FP64). Names: "x","y","z","xi","XPara0","XPara2","YPara0","YPara2",
 * "XiF3".."XiF18","Q3","Q4","Q15","Q16", BFL weight tables "XBFL37"... (idx = 0..6).
 * Returns the element count in *count. */
ISLBM_API int islbm_host_table(const islbm_params *p, const char *name, int idx, double *out, size_t cap, size_t *count);
ISLBM_API int islbm_host_table_int(const islbm_params *p, const char *name, int *out, size_t cap, size_t *count);

#ifdef __cplusplus
}
#endif
#endif
