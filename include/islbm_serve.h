/* islbm_serve.h - serving loop over many periodic-hill solves on one GPU.
 *
 * The reference has no counterpart: it runs one compile-time grid per process
 * (main loop around Launch_CollisionStreaming, C/evolution.h:842, with the controller of
 * Launch_ModifyForcingTerm, C/evolution.h:1003). This interface runs a stream of such solves
 * with different grids, Reynolds numbers, wall steepness and storage formats side by side:
 *
 *   - islbm_server_submit queues a request (the same islbm_params as islbm_init, a step cap and
 *     a convergence tolerance) and returns its id at once;
 *   - islbm_server_pump admits queued requests while the device budget allows, advances every
 *     active solve by one chunk of steps (solves of the same storage format and spanwise width
 *     share one batched step launch per step, captured once in a CUDA graph per batch), and
 *     retires solves that converged, diverged or reached their cap;
 *   - islbm_server_info / islbm_server_fields report a request's state, timings and result.
 *
 * Convergence: every steps_per_chunk steps of a solve (counted from its admission),
 * delta = sqrt(mean over nodes of |u - u_prev|^2) / Uref, with u_prev the velocity at the
 * previous check (the initial state for the first); a solve retires as converged when
 * delta < tol. A chunk ends at the next check or cap of any active solve, so a check always
 * spans exactly steps_per_chunk steps; a solve that reaches its cap between checks retires as
 * capped.
 * A request whose memory alone exceeds the budget is rejected. Results are identical to running
 * the same parameters alone through islbm_init/islbm_step: the batched launch applies the same
 * per-solve arithmetic and the same tile decomposition.
 *
 * One thread drives a server; the calls are not thread-safe on one server.
 */
#ifndef ISLBM_SERVE_H
#define ISLBM_SERVE_H

#include "islbm.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef enum islbm_solve_status {
    ISLBM_SOLVE_QUEUED = 0,
    ISLBM_SOLVE_ACTIVE = 1,
    ISLBM_SOLVE_CONVERGED = 2,
    ISLBM_SOLVE_CAPPED = 3,      /* reached max_steps before converging */
    ISLBM_SOLVE_DIVERGED = 4,    /* non-finite state, or delta above 1000 (on the way to overflow) */
    ISLBM_SOLVE_REJECTED = 5     /* could not be set up (memory, parameters) */
} islbm_solve_status;

typedef struct islbm_solve_info {
    long long id;
    int status;                  /* islbm_solve_status */
    long long steps;             /* steps taken */
    long long nodes;             /* NX*NY*NZ */
    double delta;                /* last convergence measure (-1 before the first check) */
    double force;                /* body force at retirement */
    double t_submit, t_admit, t_done;   /* seconds since the server was created */
} islbm_solve_info;

typedef struct islbm_server islbm_server;

/* hbm_budget_bytes = 0 selects 150 GiB; steps_per_chunk = steps between convergence checks. */
ISLBM_API int islbm_server_create(int device, size_t hbm_budget_bytes, int steps_per_chunk, islbm_server **out);
/* keep_fields != 0 copies rho,u,v,w to host memory at retirement for islbm_server_fields. */
ISLBM_API int islbm_server_submit(islbm_server *s, const islbm_params *p, long long max_steps, double tol,
                                  int keep_fields, long long *id);
/* One scheduling round (admit, one chunk for every active solve, retire). Blocks until the chunk
 * is done. n_active/n_queued (optional) receive the counts after the round. */
ISLBM_API int islbm_server_pump(islbm_server *s, int *n_active, int *n_queued);
ISLBM_API int islbm_server_info(islbm_server *s, long long id, islbm_solve_info *out);
/* Unique-node layout, NX*NY*NZ values each; any pointer may be NULL. Works while active, and
 * after retirement when the request was submitted with keep_fields. */
ISLBM_API int islbm_server_fields(islbm_server *s, long long id, double *rho, double *u, double *v, double *w);
/* updates: lattice-node updates so far; busy_seconds: time spent inside islbm_server_pump. */
ISLBM_API int islbm_server_stats(islbm_server *s, long long *updates, double *busy_seconds, size_t *bytes_in_use);
ISLBM_API int islbm_server_destroy(islbm_server *s);

#ifdef __cplusplus
}
#endif
#endif
