/* islbm_host.c - a C11 host program of the C ABI, compiled by the tests with gcc against
 * include/islbm.h and linked to libislbm_gb300.so.
 *
 *   islbm_host layout
 *       prints sizeof and every member offset of islbm_params and islbm_solve_info, one
 *       "name value" line each (compared with the ctypes mirror of islbm.py; no GPU needed);
 *   islbm_host run <out.bin> <steps> <precision> <Re>
 *       the reference main loop through the library, as in the integration notes: a 64x32x48
 *       hill solve from the seeded perturbed start, islbm_step in chunks of 100 steps with islbm_fields in
 *       the reference layout after each chunk (the mass-check cadence of the reference's
 *       main.cu), then writes rho, u, v, w (NX6*NYD6*NZ6 doubles each) and the body force.
 */
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "islbm.h"
#include "islbm_serve.h"

#define P_FIELD(m) printf("islbm_params.%s %zu\n", #m, offsetof(islbm_params, m))
#define I_FIELD(m) printf("islbm_solve_info.%s %zu\n", #m, offsetof(islbm_solve_info, m))

static int layout(void) {
    printf("islbm_params %zu\n", sizeof(islbm_params));
    P_FIELD(NX); P_FIELD(NY); P_FIELD(NZ); P_FIELD(LX); P_FIELD(LY); P_FIELD(LZ); P_FIELD(CFL); P_FIELD(LXi);
    P_FIELD(Re); P_FIELD(Uref); P_FIELD(NDTFRC); P_FIELD(precision); P_FIELD(les_cs); P_FIELD(alpha);
    P_FIELD(init_mode); P_FIELD(seed); P_FIELD(perturb); P_FIELD(mass_interval); P_FIELD(bfl_mode);
    P_FIELD(device); P_FIELD(kernel); P_FIELD(hbm_budget_bytes); P_FIELD(geometry);
    printf("islbm_solve_info %zu\n", sizeof(islbm_solve_info));
    I_FIELD(id); I_FIELD(status); I_FIELD(steps); I_FIELD(nodes); I_FIELD(delta); I_FIELD(force);
    I_FIELD(t_submit); I_FIELD(t_admit); I_FIELD(t_done);
    return 0;
}

static int run(const char *path, int loop, int precision, double Re) {
    islbm_params p;
    islbm_default_params(&p);              /* variables.h defaults, 64x32x48 hill */
    p.NX = 32; p.NY = 64; p.NZ = 48;        /* the old compile-time grid */
    p.Re = Re; p.Uref = 0.05; p.NDTFRC = 100;
    p.precision = precision;                /* ISLBM_FP64: the reference's arithmetic */
    p.init_mode = 1;                        /* v = Uref + 1 % seeded noise (0: rest state of InitialUsingDftFunc) */

    islbm_handle *h;
    int st = islbm_init(&p, &h);
    if (st != ISLBM_OK) { fprintf(stderr, "islbm_init: %s\n", islbm_status_string(st)); return 1; }

    const size_t nref = (size_t)(p.NX + 7)*(p.NY + 7)*(p.NZ + 6);   /* NX6 * NYD6 * NZ6 */
    double *rho_h_p = malloc(nref*sizeof(double)), *u_h_p = malloc(nref*sizeof(double));
    double *v_h_p = malloc(nref*sizeof(double)), *w_h_p = malloc(nref*sizeof(double));
    if (!rho_h_p || !u_h_p || !v_h_p || !w_h_p) { fprintf(stderr, "out of host memory\n"); return 1; }

    for (int step = 0; step < loop && st == ISLBM_OK; step += 100) {
        const int n = loop - step < 100 ? loop - step : 100;
        st = islbm_step(h, n);                                                    /* n x Launch_CollisionStreaming */
        if (st == ISLBM_OK) st = islbm_fields(h, rho_h_p, u_h_p, v_h_p, w_h_p, ISLBM_LAYOUT_REFERENCE);   /* SendDataToCPU */
    }
    double force = 0.0, rho_modify = 0.0;
    long long steps = 0;
    if (st == ISLBM_OK) st = islbm_get_scalars(h, &force, &rho_modify, &steps);
    if (st != ISLBM_OK) { fprintf(stderr, "step loop: %s\n", islbm_status_string(st)); islbm_destroy(h); return 1; }

    FILE *f = fopen(path, "wb");
    if (!f) { perror(path); islbm_destroy(h); return 1; }
    const double *outs[4] = {rho_h_p, u_h_p, v_h_p, w_h_p};
    for (int m = 0; m < 4; m++) fwrite(outs[m], sizeof(double), nref, f);
    fwrite(&force, sizeof(double), 1, f);
    fclose(f);
    printf("steps %lld force %.17g\n", steps, force);
    free(rho_h_p); free(u_h_p); free(v_h_p); free(w_h_p);
    return islbm_destroy(h) == ISLBM_OK ? 0 : 1;
}

int main(int argc, char **argv) {
    if (argc >= 2 && strcmp(argv[1], "layout") == 0) return layout();
    if (argc >= 6 && strcmp(argv[1], "run") == 0) return run(argv[2], atoi(argv[3]), atoi(argv[4]), atof(argv[5]));
    fprintf(stderr, "usage: %s layout | run <out.bin> <steps> <precision> <Re>\n", argv[0]);
    return 2;
}
