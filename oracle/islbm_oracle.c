/* CPU oracle for the ISLBM periodic-hill step (test infrastructure only; see islbm_oracle.h).
 *
 * Every function restates one piece of the reference, in the same floating-point
 * operation order, so that with -ffp-contract=off it reproduces the reference's own
 * arithmetic bit for bit (checked against the reference compiled for host cores).
 * Reference paths are relative to the solver directory `筆記：金的code/0.可更改的code/`.
 *
 * Two additions have no counterpart in the reference code and are marked where they occur:
 * the Smagorinsky closure (specified only in the LES notes, `筆記：LES_LBM/2.Hou et al.
 * (1996).tex:495-520`) and the hill-steepness factor alpha (alpha = 1 is the reference hill).
 */
#include "islbm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NQ 19

struct ora {
    ora_params p;
    int NX, NY, NZ, NX6, NYD6, NZ6;
    double LX, LY, LZ, CFL, LXi, minSize, dt, tau, niu, Uref, Re, a_nonuni;
    double *x, *y, *z, *xi;
    double *XP0[7], *XP2[7], *YP0[7], *YP2[7];
    double *XiT[8][7];                  /* XiParaF3,4,5,6,15,16,17,18 */
    int *bfl[4];                        /* BFLReqF3, F4, F15, F16 */
    double *Q[4];
    double *XB37[7], *XB38[7], *YB378[7], *XiB378[7];
    double *XB49[7], *XB410[7], *YB4910[7], *XiB4910[7];
    double *YB15[7], *XiB15[7], *YB16[7], *XiB16[7];
    double *f[2][NQ];
    double *rho, *u, *v, *w;
    double *ub_avg;
    double force, rho_modify;
    long steps;
    int cur;
    double M[NQ][NQ], Mi[NQ][NQ];
};

enum { XI3 = 0, XI4, XI5, XI6, XI15, XI16, XI17, XI18 };

/* D3Q19 velocity set in the reference's order (C/initialization.h:7-9). */
static const int E[NQ][3] = {{0,0,0},{1,0,0},{-1,0,0},{0,1,0},{0,-1,0},{0,0,1},{0,0,-1},
                             {1,1,0},{-1,1,0},{1,-1,0},{-1,-1,0},{1,0,1},{-1,0,1},{1,0,-1},
                             {-1,0,-1},{0,1,1},{0,-1,1},{0,1,-1},{0,-1,-1}};

/* Moment basis of C/MRT_Matrix.h:27-46 (d'Humieres et al. 2002 ordering), generated from its
 * defining polynomials in e; the inverse (C/MRT_Matrix.h:50-68) is M^T diag(1/|row|^2),
 * exact because the rows are orthogonal. */
static void build_mrt(double M[NQ][NQ], double Mi[NQ][NQ]) {
    for (int q = 0; q < NQ; q++) {
        const int ex = E[q][0], ey = E[q][1], ez = E[q][2];
        const int e2 = ex*ex + ey*ey + ez*ez;
        const int row[NQ] = {1, 19*e2 - 30, (21*e2*e2 - 53*e2 + 24)/2, ex, (5*e2 - 9)*ex, ey, (5*e2 - 9)*ey,
                             ez, (5*e2 - 9)*ez, 3*ex*ex - e2, (3*e2 - 5)*(3*ex*ex - e2), ey*ey - ez*ez,
                             (3*e2 - 5)*(ey*ey - ez*ez), ex*ey, ey*ez, ex*ez, (ey*ey - ez*ez)*ex,
                             (ez*ez - ex*ex)*ey, (ex*ex - ey*ey)*ez};
        for (int c = 0; c < NQ; c++) M[c][q] = (double)row[c];
    }
    for (int c = 0; c < NQ; c++) {
        double d = 0.0;
        for (int q = 0; q < NQ; q++) d += M[c][q]*M[c][q];
        for (int q = 0; q < NQ; q++) Mi[q][c] = M[c][q]/d;
    }
}

/* ---- geometry: C/model.h:4-68 ------------------------------------------------------ */
/* The six cubic segments of the periodic hill, evaluated at distance t from the crest. */
static double hill_seg(int s, double t) {
    switch (s) {
    case 1: return 1./28.*fmin(28., 28. + 0.006775070969851*t*28*t*28 - 0.0021245277758000*t*28*t*28*t*28);
    case 2: return 1./28.*(25.07355893131 + 0.9754803562315*t*28 - 0.1016116352781*t*28*t*28 + 0.001889794677828*t*28*t*28*t*28);
    case 3: return 1./28.*(25.79601052357 + 0.8206693007457*t*28 - 0.09055370274339*t*28*t*28 + 0.001626510569859*t*28*t*28*t*28);
    case 4: return 1./28.*(40.46435022819 - 1.379581654948*t*28 + 0.019458845041284*t*28*t*28 - 0.0002070318932190*t*28*t*28*t*28);
    case 5: return 1./28.*(17.92461334664 + 0.8743920332081*t*28 - 0.05567361123058*t*28*t*28 + 0.0006277731764683*t*28*t*28*t*28);
    default: return 1./28.*fmax(0., 56.39011190988 - 2.010520359035*t*28 + 0.01644919857549*t*28*t*28 + 0.00002674976141766*t*28*t*28*t*28);
    }
}

static const double HB[6] = {(54./28.)*(9./54.), (54./28.)*(14./54.), (54./28.)*(20./54.),
                             (54./28.)*(30./54.), (54./28.)*(40./54.), (54./28.)*(54./54.)};

static double hill_reference(double LY, double Y) {
    double Yb, model = 0.0;
    if (Y < 0.0) Yb = Y + LY; else if (Y > LY) Yb = Y - LY; else Yb = Y;
    if (Yb <= HB[0]) model = hill_seg(1, Yb);
    if (Yb > HB[0] && Yb <= HB[1]) model = hill_seg(2, Yb);
    if (Yb > HB[1] && Yb <= HB[2]) model = hill_seg(3, Yb);
    if (Yb > HB[2] && Yb <= HB[3]) model = hill_seg(4, Yb);
    if (Yb > HB[3] && Yb <= HB[4]) model = hill_seg(5, Yb);
    if (Yb > HB[4] && Yb <= HB[5]) model = hill_seg(6, Yb);
    const double t = LY - Yb;
    if (Yb < LY - HB[4] && Yb >= LY - HB[5]) model = hill_seg(6, t);
    if (Yb < LY - HB[3] && Yb >= LY - HB[4]) model = hill_seg(5, t);
    if (Yb < LY - HB[2] && Yb >= LY - HB[3]) model = hill_seg(4, t);
    if (Yb < LY - HB[1] && Yb >= LY - HB[2]) model = hill_seg(3, t);
    if (Yb < LY - HB[0] && Yb >= LY - HB[1]) model = hill_seg(2, t);
    if (Yb >= LY - HB[0]) model = hill_seg(1, t);
    return model;
}

/* Steepness extension (not in the reference): the footprint is stretched by alpha, the
 * height is kept; alpha == 1 returns the reference hill exactly. */
static double hill(const ora_t *o, double Y) {
    if (o->p.geometry == 1) return 0.0;   /* ChannelFunction, C/model.h:70-73 */
    const double alpha = o->p.alpha;
    if (alpha == 1.0) return hill_reference(o->LY, Y);
    double Yb = Y;
    if (Y < 0.0) Yb = Y + o->LY; else if (Y > o->LY) Yb = Y - o->LY;
    const double t = (Yb <= 0.5*o->LY ? Yb : o->LY - Yb)/alpha;
    int s = 0;
    for (int m = 0; m < 6; m++) if (t <= HB[m]) { s = m + 1; break; }
    if (s == 0) return 0.0;
    return hill_seg(s, t);
}

/* C/initializationTool.h:4-7 */
static double tanh_map(double L, double cell, double a, int j, int N) {
    return L/2.0 + cell/2.0 + ((L/2.0)/a)*tanh((-1.0 + 2.0*(double)(j)/(double)(N))/2.0*log((1.0 + a)/(1.0 - a)));
}

/* C/initializationTool.h:16-39 (iteration cap added; it never binds for valid meshes). */
static double nonuni_parameter(const ora_t *o) {
    const double total = o->LZ - hill(o, 0.0) - o->minSize;
    double a0 = 0.1, a1 = 1.0, mid, dx;
    int it = 0;
    do {
        mid = (a0 + a1)/2.0;
        const double x0 = tanh_map(total, o->minSize, mid, 0, o->NZ6 - 7);
        const double x1 = tanh_map(total, o->minSize, mid, 1, o->NZ6 - 7);
        dx = x1 - x0;
        if (dx - o->minSize >= 0.0) a0 = mid; else a1 = mid;
    } while (fabs(dx - o->minSize) > 1e-14 && ++it < 400);
    return mid;
}

/* C/initializationTool.h:60-79: 7-point Lagrange weights, same product order. */
static double lagrange6(double x, double xi, const double *others) {
    double r = (x - others[0])/(xi - others[0]);
    for (int m = 1; m < 6; m++) { r = r*(x - others[m]); r = r/(xi - others[m]); }
    return r;
}

static void lagrange_weights(double *para[7], double pos, const double *nodes, int store, int n) {
    for (int a = 0; a < 7; a++) {
        double others[6];
        int c = 0;
        for (int b = 0; b < 7; b++) if (b != a) others[c++] = nodes[n + b];
        para[a][store] = lagrange6(pos, nodes[n + a], others);
    }
}

/* C/initialization.h:185-201 (the unused nonuniform parameter is not recomputed). */
static void xi_weights(const ora_t *o, double *para[7], double pos_z, double pos_y, int store, int k) {
    const double L = o->LZ - hill(o, pos_y) - o->minSize;
    const double pos_xi = o->LXi*(pos_z - (hill(o, pos_y) + o->minSize/2.0))/L;
    int base;
    if (k >= 3 && k <= 6) base = 3;
    else if (k >= o->NZ6 - 7 && k <= o->NZ6 - 4) base = o->NZ6 - 10;
    else base = k - 3;
    lagrange_weights(para, pos_xi, o->xi, store, base);
}

/* C/initializationTool.h:81-87 */
static int bfl_needed(const ora_t *o, double Y, double Z) { return hill(o, Y) > Z ? 1 : 0; }

/* C/initializationTool.h:88-105 */
static double delta_horizontal(const ora_t *o, double z_target, double y_large, double y_small, double y_point) {
    double t0 = y_large, t1 = y_small, mid;
    int it = 0;
    do {
        mid = (t0 + t1)/2.0;
        if (hill(o, mid) >= z_target) t0 = mid; else t1 = mid;
    } while (fabs(hill(o, mid) - z_target) > 1e-13 && ++it < 400);
    return o->minSize - 2.0*fabs(y_point - mid);
}

/* C/initializationTool.h:125-152 (the outer fabs of a comparison is kept: it is a no-op). */
static double delta_45(const ora_t *o, double z_pnt, double y_pnt, double y_zdom, double y_ydom) {
    double t0 = y_zdom, t1 = y_ydom, mid;
    int it = 0;
    do {
        mid = (t0 + t1)/2.0;
        if (fabs((double)(fabs(hill(o, mid) - z_pnt) > fabs(mid - y_pnt)))) t0 = mid; else t1 = mid;
    } while (fabs(fabs(hill(o, mid) - z_pnt) - fabs(mid - y_pnt)) > 1e-13 && ++it < 400);
    return o->minSize - 2.0*fabs(y_pnt - mid);
}

static double *dalloc(size_t n) { return (double *)calloc(n ? n : 1, sizeof(double)); }

static void precompute(ora_t *o) {
    const int NX6 = o->NX6, NYD6 = o->NYD6, NZ6 = o->NZ6;
    const double ms = o->minSize;
    /* GenerateMesh_X / _Y (C/initialization.h:51-108), jp = 1 */
    const double dx = o->LX/(double)(NX6 - 2*3 - 1);
    for (int i = 0; i < NX6; i++) o->x[i] = dx*((double)(i - 3));
    const double dy = o->LY/(double)((o->NY + 7) - 2*3 - 1);
    for (int j = 0; j < NYD6; j++) o->y[j] = dy*((double)(j - 3));
    /* GenerateMesh_Z (C/initialization.h:110-137) */
    o->a_nonuni = nonuni_parameter(o);
    for (int j = 0; j < NYD6; j++) {
        const double total = o->LZ - hill(o, o->y[j]) - ms;
        for (int k = 3; k < NZ6 - 3; k++)
            o->z[j*NZ6 + k] = tanh_map(total, ms, o->a_nonuni, k - 3, NZ6 - 7) + hill(o, o->y[j]);
        o->z[j*NZ6 + 2] = hill(o, o->y[j]);
        o->z[j*NZ6 + (NZ6 - 3)] = o->LZ;
    }
    for (int k = 3; k < NZ6 - 3; k++) o->xi[k] = tanh_map(o->LXi, ms, o->a_nonuni, k - 3, NZ6 - 7) - ms/2.0;
    /* GetIntrplParameter_X / _Y (C/initialization.h:203-229) */
    for (int i = 3; i < NX6 - 3; i++) {
        lagrange_weights(o->XP0, o->x[i] - ms, o->x, i, i - 3);
        lagrange_weights(o->XP2, o->x[i] + ms, o->x, i, i - 3);
    }
    for (int j = 3; j < NYD6 - 3; j++) {
        lagrange_weights(o->YP0, o->y[j] - ms, o->y, j, j - 3);
        lagrange_weights(o->YP2, o->y[j] + ms, o->y, j, j - 3);
    }
    /* GetIntrplParameter_Xi (C/initialization.h:231-243) */
    for (int j = 3; j < NYD6 - 3; j++)
        for (int k = 3; k < NZ6 - 3; k++) {
            const double zz = o->z[j*NZ6 + k], yy = o->y[j];
            const int s = j*NZ6 + k;
            xi_weights(o, o->XiT[XI3],  zz,      yy - ms, s, k);
            xi_weights(o, o->XiT[XI4],  zz,      yy + ms, s, k);
            xi_weights(o, o->XiT[XI5],  zz - ms, yy,      s, k);
            xi_weights(o, o->XiT[XI6],  zz + ms, yy,      s, k);
            xi_weights(o, o->XiT[XI15], zz - ms, yy - ms, s, k);
            xi_weights(o, o->XiT[XI16], zz - ms, yy + ms, s, k);
            xi_weights(o, o->XiT[XI17], zz + ms, yy - ms, s, k);
            xi_weights(o, o->XiT[XI18], zz + ms, yy + ms, s, k);
        }
    /* BFLInitialization (C/initialization.h:260-333) */
    for (int k = 0; k < 2; k++)
        for (int j = 3; j < NYD6 - 3; j++) {
            const int r = k*NYD6 + j;
            const double zz = o->z[j*NZ6 + k + 3];
            o->bfl[0][r] = bfl_needed(o, o->y[j] - ms, zz);
            o->bfl[1][r] = bfl_needed(o, o->y[j] + ms, zz);
            o->bfl[2][r] = bfl_needed(o, o->y[j] - ms, zz - ms);
            o->bfl[3][r] = bfl_needed(o, o->y[j] + ms, zz - ms);
        }
    const double xm = o->x[NX6/2];
    for (int k = 0; k < 2; k++)
        for (int j = 3; j < NYD6 - 3; j++) {
            const int r = k*NYD6 + j;
            const double zz = o->z[j*NZ6 + k + 3], yy = o->y[j];
            double delta;
            if (o->bfl[0][r] == 1) {
                delta = delta_horizontal(o, zz, yy - ms, yy, yy);
                o->Q[0][r] = (ms - delta)/2.0/ms;
                lagrange_weights(o->XB38, xm - delta, o->x, r, NX6/2 - 3);
                lagrange_weights(o->XB37, xm + delta, o->x, r, NX6/2 - 3);
                lagrange_weights(o->YB378, yy + delta, o->y, r, j - 3);
                xi_weights(o, o->XiB378, zz, yy + delta, r, k + 3);
            }
            if (o->bfl[1][r] == 1) {
                delta = delta_horizontal(o, zz, yy + ms, yy, yy);
                o->Q[1][r] = (ms - delta)/2.0/ms;
                lagrange_weights(o->XB49, xm + delta, o->x, r, NX6/2 - 3);
                lagrange_weights(o->XB410, xm - delta, o->x, r, NX6/2 - 3);
                lagrange_weights(o->YB4910, yy - delta, o->y, r, j - 3);
                xi_weights(o, o->XiB4910, zz, yy - delta, r, k + 3);
            }
            if (o->bfl[2][r] == 1) {
                delta = delta_45(o, zz, yy, yy, yy - ms);
                o->Q[2][r] = (ms - delta)/2.0/ms;
                lagrange_weights(o->YB15, yy + delta, o->y, r, j - 3);
                xi_weights(o, o->XiB15, zz + delta, yy + delta, r, k + 3);
            }
            if (o->bfl[3][r] == 1) {
                delta = delta_45(o, zz, yy, yy, yy + ms);
                o->Q[3][r] = (ms - delta)/2.0/ms;
                lagrange_weights(o->YB16, yy - delta, o->y, r, j - 3);
                xi_weights(o, o->XiB16, zz + delta, yy - delta, r, k + 3);
            }
        }
}

/* Counter-based perturbation: r = splitmix64(seed + golden*(3*node + comp + 1)) -> [-1, 1). */
static double unit_noise(unsigned long long seed, unsigned long long node, int comp) {
    unsigned long long z = seed + 0x9E3779B97F4A7C15ULL*(3ULL*node + (unsigned long long)comp + 1ULL);
    z = (z ^ (z >> 30))*0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27))*0x94D049BB133111EBULL;
    z = z ^ (z >> 31);
    return (double)(z >> 11)*(1.0/9007199254740992.0)*2.0 - 1.0;
}

/* InitialUsingDftFunc (C/initialization.h:6-49); mode 1 replaces the rest state by the
 * perturbed bulk flow and reuses the same equilibrium expression. */
static void initial_state(ora_t *o) {
    static const double Wt[NQ] = {(1.0/3.0),(1.0/18.0),(1.0/18.0),(1.0/18.0),(1.0/18.0),(1.0/18.0),(1.0/18.0),
                                  (1.0/36.0),(1.0/36.0),(1.0/36.0),(1.0/36.0),(1.0/36.0),(1.0/36.0),(1.0/36.0),
                                  (1.0/36.0),(1.0/36.0),(1.0/36.0),(1.0/36.0),(1.0/36.0)};
    const int NX6 = o->NX6, NYD6 = o->NYD6, NZ6 = o->NZ6;
    const double ub = o->p.ub, amp = o->p.amp;
    for (int k = 0; k < NZ6; k++)
        for (int j = 0; j < NYD6; j++)
            for (int i = 0; i < NX6; i++) {
                const size_t index = (size_t)j*NX6*NZ6 + (size_t)k*NX6 + i;
                double rr = 1.0, uu = 0.0, vv = 0.0, ww = 0.0;
                if (o->p.init_mode == 1) {
                    const int xu = ((i - 3) % o->NX + o->NX) % o->NX, yu = ((j - 3) % o->NY + o->NY) % o->NY;
                    int zu = k - 3; if (zu < 0) zu = 0; if (zu > o->NZ - 1) zu = o->NZ - 1;
                    const unsigned long long node = ((unsigned long long)zu*o->NY + yu)*o->NX + xu;
                    uu = ub*amp*unit_noise(o->p.seed, node, 0);
                    vv = ub + ub*amp*unit_noise(o->p.seed, node, 1);
                    ww = ub*amp*unit_noise(o->p.seed, node, 2);
                }
                o->rho[index] = rr; o->u[index] = uu; o->v[index] = vv; o->w[index] = ww;
                const double udot = uu*uu + vv*vv + ww*ww;
                o->f[0][0][index] = Wt[0]*rr*(1.0 - 1.5*udot);
                for (int q = 1; q < NQ; q++) {
                    const double eu = (double)E[q][0]*uu + (double)E[q][1]*vv + (double)E[q][2]*ww;
                    o->f[0][q][index] = Wt[q]*rr*(1.0 + 3.0*eu + 4.5*eu*eu - 1.5*udot);
                }
            }
    for (int q = 0; q < NQ; q++) memcpy(o->f[1][q], o->f[0][q], (size_t)NX6*NYD6*NZ6*sizeof(double));
    o->force = (8.0*o->niu*o->Uref)/(o->LZ*o->LZ)*5.0;
}

/* ---- the step: C/evolution.h:358-684 --------------------------------------------------- */
static inline double i7(const double *f, size_t base, size_t stride, const double *const w[7], int wi) {
    /* Intrpl7 (C/interpolationHillISLBM.h:4-7): left-to-right sum of value*weight */
    double s = f[base]*w[0][wi];
    for (int a = 1; a < 7; a++) s = s + f[base + a*stride]*w[a][wi];
    return s;
}

static inline double interp_xy_xi(const double *f, size_t idx, size_t nline, size_t nface,
                                  double *const xw[7], int ix, double *const yw[7], int iy,
                                  double *const zw[7], int iz) {
    /* X_Y_XI_Intrpl7: x innermost, then y, then xi (C/interpolationHillISLBM.h:68-135) */
    double outer = 0.0;
    for (int c = 0; c < 7; c++) {
        double mid = 0.0;
        for (int b = 0; b < 7; b++) {
            const double in = i7(f, idx + b*nface + c*nline, 1, (const double *const *)xw, ix);
            mid = (b == 0) ? in*yw[0][iy] : mid + in*yw[b][iy];
        }
        outer = (c == 0) ? mid*zw[0][iz] : outer + mid*zw[c][iz];
    }
    return outer;
}

static inline double interp_x_xi(const double *f, size_t idx, size_t nline,
                                 double *const xw[7], int ix, double *const zw[7], int iz) {
    /* X_XI_Intrpl7 (C/interpolationHillISLBM.h:137-148) */
    double outer = 0.0;
    for (int c = 0; c < 7; c++) {
        const double in = i7(f, idx + c*nline, 1, (const double *const *)xw, ix);
        outer = (c == 0) ? in*zw[0][iz] : outer + in*zw[c][iz];
    }
    return outer;
}

static inline double interp_y_xi(const double *f, size_t idx, size_t nline, size_t nface,
                                 double *const yw[7], int iy, double *const zw[7], int iz) {
    /* Y_XI_Intrpl7: y inner, xi outer (C/interpolationHillISLBM.h:150-161) */
    double outer = 0.0;
    for (int c = 0; c < 7; c++) {
        const double in = i7(f, idx + c*nline, nface, (const double *const *)yw, iy);
        outer = (c == 0) ? in*zw[0][iz] : outer + in*zw[c][iz];
    }
    return outer;
}

static inline double interp_xi_y(const double *f, size_t idx, size_t nline, size_t nface,
                                 double *const yw[7], int iy, double *const zw[7], int iz) {
    /* F3_Intrpl7 / F4_Intrpl7: xi inner, y outer (C/interpolationHillISLBM.h:22-58) */
    double outer = 0.0;
    for (int b = 0; b < 7; b++) {
        const double in = i7(f, idx + b*nface, nline, (const double *const *)zw, iz);
        outer = (b == 0) ? in*yw[0][iy] : outer + in*yw[b][iy];
    }
    return outer;
}

static double zero_col[1] = {0.0};

static void node_update(ora_t *o, const double *const *fo, double *const *fn, int i, int j, int k) {
    const int NX6 = o->NX6, NYD6 = o->NYD6, NZ6 = o->NZ6;
    const size_t nface = (size_t)NX6*NZ6, nline = (size_t)NX6;
    const size_t index = (size_t)j*nface + (size_t)k*nline + i;
    int cell_z = k - 3;
    if (k <= 6) cell_z = 3;
    if (k >= NZ6 - 7) cell_z = NZ6 - 10;
    const int ixi = j*NZ6 + k;
    double F[NQ];
    const size_t row_x = (size_t)j*nface + (size_t)k*nline + (i - 3);
    const size_t col_z = (size_t)j*nface + (size_t)cell_z*nline + i;
    const size_t slab_y = (size_t)(j - 3)*nface + (size_t)cell_z*nline + i;
    const size_t cube = (size_t)(j - 3)*nface + (size_t)cell_z*nline + (i - 3);
    const size_t plane_xz = (size_t)j*nface + (size_t)cell_z*nline + (i - 3);

    F[0] = fo[0][index];
    F[1] = i7(fo[1], row_x, 1, (const double *const *)o->XP0, i);
    F[2] = i7(fo[2], row_x, 1, (const double *const *)o->XP2, i);
    F[3] = interp_xi_y(fo[3], slab_y, nline, nface, o->YP0, j, o->XiT[XI3], ixi);
    F[4] = interp_xi_y(fo[4], slab_y, nline, nface, o->YP2, j, o->XiT[XI4], ixi);
    F[5] = i7(fo[5], col_z, nline, (const double *const *)o->XiT[XI5], ixi);
    F[6] = i7(fo[6], col_z, nline, (const double *const *)o->XiT[XI6], ixi);
    F[7]  = interp_xy_xi(fo[7],  cube, nline, nface, o->XP0, i, o->YP0, j, o->XiT[XI3], ixi);
    F[8]  = interp_xy_xi(fo[8],  cube, nline, nface, o->XP2, i, o->YP0, j, o->XiT[XI3], ixi);
    F[9]  = interp_xy_xi(fo[9],  cube, nline, nface, o->XP0, i, o->YP2, j, o->XiT[XI4], ixi);
    F[10] = interp_xy_xi(fo[10], cube, nline, nface, o->XP2, i, o->YP2, j, o->XiT[XI4], ixi);
    F[11] = interp_x_xi(fo[11], plane_xz, nline, o->XP0, i, o->XiT[XI5], ixi);
    F[12] = interp_x_xi(fo[12], plane_xz, nline, o->XP2, i, o->XiT[XI5], ixi);
    F[13] = interp_x_xi(fo[13], plane_xz, nline, o->XP0, i, o->XiT[XI6], ixi);
    F[14] = interp_x_xi(fo[14], plane_xz, nline, o->XP2, i, o->XiT[XI6], ixi);
    F[15] = interp_y_xi(fo[15], slab_y, nline, nface, o->YP0, j, o->XiT[XI15], ixi);
    F[16] = interp_y_xi(fo[16], slab_y, nline, nface, o->YP2, j, o->XiT[XI16], ixi);
    F[17] = interp_y_xi(fo[17], slab_y, nline, nface, o->YP0, j, o->XiT[XI17], ixi);
    F[18] = interp_y_xi(fo[18], slab_y, nline, nface, o->YP2, j, o->XiT[XI18], ixi);

    /* half-way bounce-back at both walls (C/evolution.h:482-496) */
    if (k == 3) { F[5] = fo[6][index]; F[11] = fo[14][index]; F[12] = fo[13][index]; F[15] = fo[18][index]; F[16] = fo[17][index]; }
    if (k == NZ6 - 4) { F[6] = fo[5][index]; F[13] = fo[12][index]; F[14] = fo[11][index]; F[17] = fo[16][index]; F[18] = fo[15][index]; }

    /* BFL curved-wall rows k = 3, 4 (C/evolution.h:505-572) */
    if (k == 3 || k == 4) {
        const int r = (k - 3)*NYD6 + j;
        /* table index of the x and y weights: the reference's active code passes i and j
         * (C/evolution.h:525-527); bfl_mode 1 uses the row index r for all three. */
        const int ix = o->p.bfl_mode ? r : i, iy = o->p.bfl_mode ? r : j;
        const size_t bslab = (size_t)(j - 3)*nface + (size_t)3*nline + i;
        const size_t bcube = (size_t)(j - 3)*nface + (size_t)3*nline + (i - 3);
        double *zx[7];
        int ixx = ix;
        if (ix >= 2*NYD6) { for (int a = 0; a < 7; a++) zx[a] = zero_col; ixx = 0; }
        if (o->bfl[0][r] == 1) {
            const double q = o->Q[0][r];
            if (q > 0.5) {
                F[3] = (1/(2*q))*fo[4][index] + ((2*q - 1)/(2*q))*fo[3][index];
                F[7] = (1/(2*q))*fo[10][index] + ((2*q - 1)/(2*q))*fo[7][index];
                F[8] = (1/(2*q))*fo[9][index] + ((2*q - 1)/(2*q))*fo[8][index];
            }
            if (q < 0.5) {
                F[3] = interp_y_xi(fo[4], bslab, nline, nface, o->YB378, iy, o->XiB378, r);
                F[7] = interp_xy_xi(fo[10], bcube, nline, nface, ix >= 2*NYD6 ? zx : o->XB37, ixx, o->YB378, iy, o->XiB378, r);
                F[8] = interp_xy_xi(fo[9], bcube, nline, nface, ix >= 2*NYD6 ? zx : o->XB38, ixx, o->YB378, iy, o->XiB378, r);
            }
        }
        if (o->bfl[1][r] == 1) {
            const double q = o->Q[1][r];
            if (q > 0.5) {
                F[4] = (1/(2*q))*fo[3][index] + ((2*q - 1)/(2*q))*fo[4][index];
                F[9] = (1/(2*q))*fo[8][index] + ((2*q - 1)/(2*q))*fo[9][index];
                F[10] = (1/(2*q))*fo[7][index] + ((2*q - 1)/(2*q))*fo[10][index];
            }
            if (q < 0.5) {
                F[4] = interp_y_xi(fo[3], bslab, nline, nface, o->YB4910, iy, o->XiB4910, r);
                F[9] = interp_xy_xi(fo[8], bcube, nline, nface, ix >= 2*NYD6 ? zx : o->XB49, ixx, o->YB4910, iy, o->XiB4910, r);
                F[10] = interp_xy_xi(fo[7], bcube, nline, nface, ix >= 2*NYD6 ? zx : o->XB410, ixx, o->YB4910, iy, o->XiB4910, r);
            }
        }
        if (o->bfl[2][r] == 1) {
            const double q = o->Q[2][r];
            if (q > 0.5) F[15] = (1/(2*q))*fo[18][index] + ((2*q - 1)/(2*q))*fo[15][index];
            if (q < 0.5) F[15] = interp_y_xi(fo[18], bslab, nline, nface, o->YB15, iy, o->XiB15, r);
        }
        if (o->bfl[3][r] == 1) {
            const double q = o->Q[3][r];
            if (q > 0.5) F[16] = (1/(2*q))*fo[17][index] + ((2*q - 1)/(2*q))*fo[16][index];
            if (q < 0.5) F[16] = interp_y_xi(fo[17], bslab, nline, nface, o->YB16, iy, o->XiB16, r);
        }
    }

    F[0] = F[0] + o->rho_modify;   /* C/evolution.h:597 */

    /* macroscopic quantities and equilibrium (C/evolution.h:600-626) */
    double rho_s = F[0];
    for (int q = 1; q < NQ; q++) rho_s = rho_s + F[q];
    const double u1 = (F[1] + F[7] + F[9] + F[11] + F[13] - (F[2] + F[8] + F[10] + F[12] + F[14]))/rho_s;
    const double v1 = (F[3] + F[7] + F[8] + F[15] + F[17] - (F[4] + F[9] + F[10] + F[16] + F[18]))/rho_s;
    const double w1 = (F[5] + F[11] + F[12] + F[15] + F[16] - (F[6] + F[13] + F[14] + F[17] + F[18]))/rho_s;
    const double udot = u1*u1 + v1*v1 + w1*w1;
    double Feq[NQ];
    Feq[0] = (1./3.)*rho_s*(1.0 - 1.5*udot);
    Feq[1] = (1./18.)*rho_s*(1.0 + 3.0*u1 + 4.5*u1*u1 - 1.5*udot);
    Feq[2] = (1./18.)*rho_s*(1.0 - 3.0*u1 + 4.5*u1*u1 - 1.5*udot);
    Feq[3] = (1./18.)*rho_s*(1.0 + 3.0*v1 + 4.5*v1*v1 - 1.5*udot);
    Feq[4] = (1./18.)*rho_s*(1.0 - 3.0*v1 + 4.5*v1*v1 - 1.5*udot);
    Feq[5] = (1./18.)*rho_s*(1.0 + 3.0*w1 + 4.5*w1*w1 - 1.5*udot);
    Feq[6] = (1./18.)*rho_s*(1.0 - 3.0*w1 + 4.5*w1*w1 - 1.5*udot);
    Feq[7] = (1./36.)*rho_s*(1.0 + 3.0*(u1 + v1) + 4.5*(u1 + v1)*(u1 + v1) - 1.5*udot);
    Feq[8] = (1./36.)*rho_s*(1.0 + 3.0*(-u1 + v1) + 4.5*(-u1 + v1)*(-u1 + v1) - 1.5*udot);
    Feq[9] = (1./36.)*rho_s*(1.0 + 3.0*(u1 - v1) + 4.5*(u1 - v1)*(u1 - v1) - 1.5*udot);
    Feq[10] = (1./36.)*rho_s*(1.0 + 3.0*(-u1 - v1) + 4.5*(-u1 - v1)*(-u1 - v1) - 1.5*udot);
    Feq[11] = (1./36.)*rho_s*(1.0 + 3.0*(u1 + w1) + 4.5*(u1 + w1)*(u1 + w1) - 1.5*udot);
    Feq[12] = (1./36.)*rho_s*(1.0 + 3.0*(-u1 + w1) + 4.5*(-u1 + w1)*(-u1 + w1) - 1.5*udot);
    Feq[13] = (1./36.)*rho_s*(1.0 + 3.0*(u1 - w1) + 4.5*(u1 - w1)*(u1 - w1) - 1.5*udot);
    Feq[14] = (1./36.)*rho_s*(1.0 + 3.0*(-u1 - w1) + 4.5*(-u1 - w1)*(-u1 - w1) - 1.5*udot);
    Feq[15] = (1./36.)*rho_s*(1.0 + 3.0*(v1 + w1) + 4.5*(v1 + w1)*(v1 + w1) - 1.5*udot);
    Feq[16] = (1./36.)*rho_s*(1.0 + 3.0*(-v1 + w1) + 4.5*(-v1 + w1)*(-v1 + w1) - 1.5*udot);
    Feq[17] = (1./36.)*rho_s*(1.0 + 3.0*(v1 - w1) + 4.5*(v1 - w1)*(v1 - w1) - 1.5*udot);
    Feq[18] = (1./36.)*rho_s*(1.0 + 3.0*(-v1 - w1) + 4.5*(-v1 - w1)*(-v1 - w1) - 1.5*udot);

    /* relaxation rates (C/MRT_Matrix.h:4-23) */
    double tau_e = o->tau;
    if (o->p.les_cs > 0.0) {
        /* Smagorinsky closure (not in the reference code; LES notes :495-520):
         * Q = Pi^neq : Pi^neq, |S| = (sqrt(nu0^2 + 18 C Q^(1/2)) - nu0)/(6 C), C = Cs^2,
         * tau* = tau0 + 3 C |S|, all in lattice units (filter width = lattice spacing). */
        double pxx = 0, pyy = 0, pzz = 0, pxy = 0, pyz = 0, pxz = 0;
        for (int q = 1; q < NQ; q++) {
            const double d = F[q] - Feq[q];
            pxx += E[q][0]*E[q][0]*d; pyy += E[q][1]*E[q][1]*d; pzz += E[q][2]*E[q][2]*d;
            pxy += E[q][0]*E[q][1]*d; pyz += E[q][1]*E[q][2]*d; pxz += E[q][0]*E[q][2]*d;
        }
        const double Qn = pxx*pxx + pyy*pyy + pzz*pzz + 2.0*(pxy*pxy + pyz*pyz + pxz*pxz);
        const double C = o->p.les_cs*o->p.les_cs;
        const double nu0 = (o->tau - 0.5)/3.0;
        const double S = (sqrt(nu0*nu0 + 18.0*C*sqrt(Qn)) - nu0)/(6.0*C);
        tau_e = o->tau + 3.0*C*S;
    }
    const double s[NQ] = {0.0, 1.19, 1.4, 0.0, 1.2, 0.0, 1.2, 0.0, 1.2, (1.0/tau_e), 1.4, (1.0/tau_e), 1.4,
                          (1.0/tau_e), (1.0/tau_e), (1.0/tau_e), 1.5, 1.5, 1.5};

    /* m = M F, meq = M Feq, F -= Mi S (m - meq) + body force (C/MRT_Process.h:4-179).
     * Terms whose matrix entry or rate is zero contribute an exact zero and are skipped. */
    double m[NQ], meq[NQ];
    for (int c = 0; c < NQ; c++) {
        double a = F[0]*o->M[c][0], b = Feq[0]*o->M[c][0];
        for (int q = 1; q < NQ; q++)
            if (o->M[c][q] != 0.0) { a = a + F[q]*o->M[c][q]; b = b + Feq[q]*o->M[c][q]; }
        m[c] = a; meq[c] = b;
    }
    const double fdt = o->force;
    for (int q = 0; q < NQ; q++) {
        double r = F[q];
        for (int c = 0; c < NQ; c++)
            if (o->Mi[q][c] != 0.0 && s[c] != 0.0) r = r - o->Mi[q][c]*s[c]*(m[c] - meq[c]);
        switch (q) {
        case 3: r = r + 1.0/6*fdt*o->dt; break;
        case 4: r = r - 1.0/6*fdt*o->dt; break;
        case 7: case 8: case 15: case 17: r = r + 1.0/12*fdt*o->dt; break;
        case 9: case 10: case 16: case 18: r = r - 1.0/12*fdt*o->dt; break;
        default: break;
        }
        fn[q][index] = r;
    }
    o->u[index] = u1; o->v[index] = v1; o->w[index] = w1; o->rho[index] = rho_s;
}

static void periodic_copy(ora_t *o, double *const *fn) {
    const int NX6 = o->NX6, NYD6 = o->NYD6, NZ6 = o->NZ6, NX = o->NX, NY = o->NY;
    const size_t nface = (size_t)NX6*NZ6;
    double *arr[NQ + 4];
    for (int q = 0; q < NQ; q++) arr[q] = fn[q];
    arr[NQ] = o->u; arr[NQ + 1] = o->v; arr[NQ + 2] = o->w; arr[NQ + 3] = o->rho;
    /* periodicUD (C/evolution.h:686-730): rows 0..2 <- +NY, rows NYD6-1-j <- -NY */
    for (int a = 0; a < NQ + 4; a++)
        for (int k = 0; k < NZ6; k++)
            for (int jj = 0; jj < 3; jj++)
                for (int i = 0; i < NX6; i++) {
                    size_t dst = (size_t)jj*nface + (size_t)k*NX6 + i;
                    arr[a][dst] = arr[a][dst + (size_t)NY*nface];
                    dst = (size_t)(NYD6 - 1 - jj)*nface + (size_t)k*NX6 + i;
                    arr[a][dst] = arr[a][dst - (size_t)NY*nface];
                }
    /* periodicSW (C/evolution.h:732-777): cols 0..2 <- +NX, cols NX6-1-i <- -NX */
    for (int a = 0; a < NQ + 4; a++)
        for (int k = 0; k < NZ6; k++)
            for (int j = 0; j < NYD6; j++)
                for (int ii = 0; ii < 3; ii++) {
                    size_t dst = (size_t)j*nface + (size_t)k*NX6 + ii;
                    arr[a][dst] = arr[a][dst + NX];
                    dst = (size_t)j*nface + (size_t)k*NX6 + (NX6 - 1 - ii);
                    arr[a][dst] = arr[a][dst - NX];
                }
}

static void one_step(ora_t *o) {
    const int NX6 = o->NX6, NYD6 = o->NYD6, NZ6 = o->NZ6;
    double *const *fo = o->f[o->cur];
    double *const *fn = o->f[1 - o->cur];
    /* AccumulateUbulk (C/evolution.h:826-840) on plane j = 0, previous step's v */
    for (int k = 3; k <= NZ6 - 4; k++)
        for (int i = 3; i <= NX6 - 4; i++) {
            const double dx = (o->x[i + 1] - o->x[i - 1])/2.0;
            const double dz = (o->z[k + 1] - o->z[k - 1])/2.0;
            o->ub_avg[k*NX6 + i] += o->v[(size_t)k*NX6 + i]*dx*dz;
        }
    /* every interior row once (C/evolution.h:55-356 and :358-684 share this body) */
#pragma omp parallel for schedule(static) collapse(2)
    for (int j = 3; j <= NYD6 - 4; j++)
        for (int k = 3; k <= NZ6 - 4; k++)
            for (int i = 3; i <= NX6 - 4; i++)
                node_update(o, (const double *const *)fo, fn, i, j, k);
    periodic_copy(o, fn);
    o->cur = 1 - o->cur;
    o->steps++;
    /* Launch_ModifyForcingTerm (C/evolution.h:1003-1042), jp = 1 */
    if (o->steps % o->p.ndtfrc == 0) {
        double ub = 0.0;
        for (int k = 3; k < NZ6 - 3; k++)
            for (int i = 3; i < NX6 - 4; i++) { ub = ub + o->ub_avg[k*NX6 + i]; o->ub_avg[k*NX6 + i] = 0.0; }
        ub = ub/(double)(o->LX*(o->LZ - 1.0))/o->p.ndtfrc;
        const double beta = fmax(0.001, 3.0/(double)o->Re);
        o->force = o->force + beta*(o->Uref - ub)*o->Uref/3.036;
    }
    /* mass correction consumed at C/evolution.h:597; rule of this project (the reference's
     * producer lives in the missing main.cu): (N - sum rho)/N for one step every K steps. */
    o->rho_modify = 0.0;
    if (o->p.mass_interval > 0 && o->steps % o->p.mass_interval == 0) {
        double mass = 0.0;
        for (int k = 3; k <= NZ6 - 4; k++)
            for (int j = 3; j <= NYD6 - 5; j++)
                for (int i = 3; i <= NX6 - 5; i++) mass += o->rho[(size_t)j*NX6*NZ6 + (size_t)k*NX6 + i];
        const double n = (double)o->NX*(double)o->NY*(double)o->NZ;
        o->rho_modify = (n - mass)/n;
    }
}

ora_t *ora_create(const ora_params *p) {
    if (!p || p->nx < 1 || p->ny < 8 || p->nz < 8 || p->ndtfrc < 1) return NULL;
    ora_t *o = (ora_t *)calloc(1, sizeof(ora_t));
    if (!o) return NULL;
    o->p = *p;
    if (o->p.alpha <= 0.0) o->p.alpha = 1.0;
    o->NX = p->nx; o->NY = p->ny; o->NZ = p->nz;
    o->NX6 = p->nx + 7; o->NYD6 = p->ny + 7; o->NZ6 = p->nz + 6;
    o->LX = p->lx; o->LY = p->ly; o->LZ = p->lz; o->CFL = p->cfl; o->LXi = p->lxi; o->Re = p->re;
    /* C/variables.h:22-23, 76, 97-101, with tau from (Re, Ub) so that Uref = Re*niu = Ub */
    o->minSize = ((o->LZ - 1.0)/(double)(o->NZ6 - 6))*o->CFL;
    o->dt = o->minSize;
    o->tau = 0.5 + 3.0*(p->ub)/((double)o->Re*o->minSize);
    o->niu = ((o->tau - 0.5)/3.0*o->dt);
    o->Uref = (o->Re*o->niu);
    build_mrt(o->M, o->Mi);
    const size_t n3 = (size_t)o->NX6*o->NYD6*o->NZ6;
    o->x = dalloc(o->NX6); o->y = dalloc(o->NYD6); o->z = dalloc((size_t)o->NYD6*o->NZ6); o->xi = dalloc(o->NZ6);
    for (int a = 0; a < 7; a++) {
        o->XP0[a] = dalloc(o->NX6); o->XP2[a] = dalloc(o->NX6);
        o->YP0[a] = dalloc(o->NYD6); o->YP2[a] = dalloc(o->NYD6);
        for (int t = 0; t < 8; t++) o->XiT[t][a] = dalloc((size_t)o->NYD6*o->NZ6);
        const size_t nb = 2*(size_t)o->NYD6;
        o->XB37[a] = dalloc(nb); o->XB38[a] = dalloc(nb); o->YB378[a] = dalloc(nb); o->XiB378[a] = dalloc(nb);
        o->XB49[a] = dalloc(nb); o->XB410[a] = dalloc(nb); o->YB4910[a] = dalloc(nb); o->XiB4910[a] = dalloc(nb);
        o->YB15[a] = dalloc(nb); o->XiB15[a] = dalloc(nb); o->YB16[a] = dalloc(nb); o->XiB16[a] = dalloc(nb);
    }
    for (int t = 0; t < 4; t++) { o->bfl[t] = (int *)calloc(2*(size_t)o->NYD6, sizeof(int)); o->Q[t] = dalloc(2*(size_t)o->NYD6); }
    for (int b = 0; b < 2; b++) for (int q = 0; q < NQ; q++) o->f[b][q] = dalloc(n3);
    o->rho = dalloc(n3); o->u = dalloc(n3); o->v = dalloc(n3); o->w = dalloc(n3);
    o->ub_avg = dalloc((size_t)o->NX6*o->NZ6);
#ifdef _OPENMP
    if (p->threads > 0) omp_set_num_threads(p->threads);
#endif
    precompute(o);
    initial_state(o);
    o->cur = 0; o->steps = 0; o->rho_modify = 0.0;
    return o;
}

void ora_destroy(ora_t *o) {
    if (!o) return;
    free(o->x); free(o->y); free(o->z); free(o->xi);
    for (int a = 0; a < 7; a++) {
        free(o->XP0[a]); free(o->XP2[a]); free(o->YP0[a]); free(o->YP2[a]);
        for (int t = 0; t < 8; t++) free(o->XiT[t][a]);
        free(o->XB37[a]); free(o->XB38[a]); free(o->YB378[a]); free(o->XiB378[a]);
        free(o->XB49[a]); free(o->XB410[a]); free(o->YB4910[a]); free(o->XiB4910[a]);
        free(o->YB15[a]); free(o->XiB15[a]); free(o->YB16[a]); free(o->XiB16[a]);
    }
    for (int t = 0; t < 4; t++) { free(o->bfl[t]); free(o->Q[t]); }
    for (int b = 0; b < 2; b++) for (int q = 0; q < NQ; q++) free(o->f[b][q]);
    free(o->rho); free(o->u); free(o->v); free(o->w); free(o->ub_avg);
    free(o);
}

int ora_step(ora_t *o, int nsteps) {
    if (!o || nsteps < 0) return -1;
    for (int s = 0; s < nsteps; s++) one_step(o);
    return 0;
}

int ora_dims(const ora_t *o, int *out) {
    out[0] = o->NX6; out[1] = o->NYD6; out[2] = o->NZ6; out[3] = o->NX; out[4] = o->NY; out[5] = o->NZ;
    return 0;
}

double ora_force(const ora_t *o) { return o->force; }
void ora_set_force(ora_t *o, double force) { o->force = force; }

double ora_scalar(const ora_t *o, const char *name) {
    if (!strcmp(name, "tau")) return o->tau;
    if (!strcmp(name, "niu")) return o->niu;
    if (!strcmp(name, "Uref")) return o->Uref;
    if (!strcmp(name, "minSize")) return o->minSize;
    if (!strcmp(name, "a")) return o->a_nonuni;
    if (!strcmp(name, "force")) return o->force;
    if (!strcmp(name, "rho_modify")) return o->rho_modify;
    if (!strcmp(name, "steps")) return (double)o->steps;
    return NAN;
}

int ora_set_f(ora_t *o, int q, const double *in) {
    if (q < 0 || q >= NQ) return -1;
    memcpy(o->f[o->cur][q], in, (size_t)o->NX6*o->NYD6*o->NZ6*sizeof(double));
    return 0;
}

long ora_get(const ora_t *o, const char *name, int idx, double *out) {
    const size_t n3 = (size_t)o->NX6*o->NYD6*o->NZ6, nb = 2*(size_t)o->NYD6, nyz = (size_t)o->NYD6*o->NZ6;
    const double *src = NULL;
    size_t cnt = 0;
    if (idx < 0 || idx > 18) return -1;
    int a = idx % 7;
    if (!strcmp(name, "f")) { src = o->f[o->cur][idx]; cnt = n3; }
    else if (!strcmp(name, "rho")) { src = o->rho; cnt = n3; }
    else if (!strcmp(name, "u")) { src = o->u; cnt = n3; }
    else if (!strcmp(name, "v")) { src = o->v; cnt = n3; }
    else if (!strcmp(name, "w")) { src = o->w; cnt = n3; }
    else if (!strcmp(name, "x")) { src = o->x; cnt = o->NX6; }
    else if (!strcmp(name, "y")) { src = o->y; cnt = o->NYD6; }
    else if (!strcmp(name, "z")) { src = o->z; cnt = nyz; }
    else if (!strcmp(name, "xi")) { src = o->xi; cnt = o->NZ6; }
    else if (!strcmp(name, "XPara0")) { src = o->XP0[a]; cnt = o->NX6; }
    else if (!strcmp(name, "XPara2")) { src = o->XP2[a]; cnt = o->NX6; }
    else if (!strcmp(name, "YPara0")) { src = o->YP0[a]; cnt = o->NYD6; }
    else if (!strcmp(name, "YPara2")) { src = o->YP2[a]; cnt = o->NYD6; }
    else if (!strcmp(name, "XiF3")) { src = o->XiT[XI3][a]; cnt = nyz; }
    else if (!strcmp(name, "XiF4")) { src = o->XiT[XI4][a]; cnt = nyz; }
    else if (!strcmp(name, "XiF5")) { src = o->XiT[XI5][a]; cnt = nyz; }
    else if (!strcmp(name, "XiF6")) { src = o->XiT[XI6][a]; cnt = nyz; }
    else if (!strcmp(name, "XiF15")) { src = o->XiT[XI15][a]; cnt = nyz; }
    else if (!strcmp(name, "XiF16")) { src = o->XiT[XI16][a]; cnt = nyz; }
    else if (!strcmp(name, "XiF17")) { src = o->XiT[XI17][a]; cnt = nyz; }
    else if (!strcmp(name, "XiF18")) { src = o->XiT[XI18][a]; cnt = nyz; }
    else if (!strcmp(name, "Q3")) { src = o->Q[0]; cnt = nb; }
    else if (!strcmp(name, "Q4")) { src = o->Q[1]; cnt = nb; }
    else if (!strcmp(name, "Q15")) { src = o->Q[2]; cnt = nb; }
    else if (!strcmp(name, "Q16")) { src = o->Q[3]; cnt = nb; }
    else if (!strcmp(name, "XBFL37")) { src = o->XB37[a]; cnt = nb; }
    else if (!strcmp(name, "XBFL38")) { src = o->XB38[a]; cnt = nb; }
    else if (!strcmp(name, "YBFL378")) { src = o->YB378[a]; cnt = nb; }
    else if (!strcmp(name, "XiBFL378")) { src = o->XiB378[a]; cnt = nb; }
    else if (!strcmp(name, "XBFL49")) { src = o->XB49[a]; cnt = nb; }
    else if (!strcmp(name, "XBFL410")) { src = o->XB410[a]; cnt = nb; }
    else if (!strcmp(name, "YBFL4910")) { src = o->YB4910[a]; cnt = nb; }
    else if (!strcmp(name, "XiBFL4910")) { src = o->XiB4910[a]; cnt = nb; }
    else if (!strcmp(name, "YBFL15")) { src = o->YB15[a]; cnt = nb; }
    else if (!strcmp(name, "XiBFL15")) { src = o->XiB15[a]; cnt = nb; }
    else if (!strcmp(name, "YBFL16")) { src = o->YB16[a]; cnt = nb; }
    else if (!strcmp(name, "XiBFL16")) { src = o->XiB16[a]; cnt = nb; }
    else if (!strcmp(name, "UbAvg")) { src = o->ub_avg; cnt = (size_t)o->NX6*o->NZ6; }
    else if (!strcmp(name, "M")) { src = &o->M[idx][0]; cnt = NQ; }
    else if (!strcmp(name, "Mi")) { src = &o->Mi[idx][0]; cnt = NQ; }
    if (!src) return -1;
    memcpy(out, src, cnt*sizeof(double));
    return (long)cnt;
}

long ora_get_int(const ora_t *o, const char *name, int *out) {
    const int *src = NULL;
    if (!strcmp(name, "BFL3")) src = o->bfl[0];
    else if (!strcmp(name, "BFL4")) src = o->bfl[1];
    else if (!strcmp(name, "BFL15")) src = o->bfl[2];
    else if (!strcmp(name, "BFL16")) src = o->bfl[3];
    if (!src) return -1;
    memcpy(out, src, 2*(size_t)o->NYD6*sizeof(int));
    return 2*(long)o->NYD6;
}
