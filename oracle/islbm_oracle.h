/* CPU oracle for the ISLBM periodic-hill step (test infrastructure only).
 *
 * A plain-C FP64 restatement of the reference's evolution step, in the reference's own
 * storage layout (NX6 x NYD6 x NZ6 with 3 ghost layers and duplicated periodic end nodes,
 * index = j*NX6*NZ6 + k*NX6 + i). It is the checker for the CUDA library: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it. Parity of this oracle
 * with the reference itself is pinned by tests/test_oracle_vs_reference.py (reference
 * compiled for host cores by oracle/ref_build.py) and by the fixtures in tests/golden/.
 */
#ifndef ISLBM_ORACLE_H
#define ISLBM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ora_params {
    int nx, ny, nz;          /* reference NX (spanwise), NY (streamwise), NZ (wall-normal) */
    double lx, ly, lz;       /* 4.5, 9.0, 3.036 */
    double cfl, lxi;         /* 0.6, 10.0 */
    double re, ub;           /* Reynolds number, bulk velocity (Uref) */
    int ndtfrc;              /* forcing-controller period */
    int init_mode;           /* 0 rest state, 1 perturbed bulk flow */
    unsigned long long seed;
    double amp;              /* perturbation amplitude relative to ub */
    int mass_interval;       /* 0 off; else rho_modify every mass_interval steps */
    int bfl_mode;            /* 0 reference table indexing, 1 corrected */
    double les_cs;           /* Smagorinsky constant, 0 = off */
    double alpha;            /* hill steepness (1 = reference hill) */
    int threads;             /* OpenMP threads, 0 = runtime default */
    int geometry;            /* 0 hill (C/model.h:4-68), 1 flat channel (ChannelFunction, C/model.h:70-73) */
} ora_params;

typedef struct ora ora_t;

ora_t *ora_create(const ora_params *p);
void ora_destroy(ora_t *o);
int ora_step(ora_t *o, int nsteps);
int ora_dims(const ora_t *o, int *out6);
double ora_force(const ora_t *o);
double ora_scalar(const ora_t *o, const char *name);
long ora_get(const ora_t *o, const char *name, int idx, double *out);
long ora_get_int(const ora_t *o, const char *name, int *out);
int ora_set_f(ora_t *o, int q, const double *in);
void ora_set_force(ora_t *o, double force);

#ifdef __cplusplus
}
#endif
#endif
