// Host FP64 precompute; see geometry.hpp for the reference functions each part follows.
// Compiled with -ffp-contract=off so the host compiler keeps the reference's rounding.
#include "geometry.hpp"

#include <cmath>
#include <cstring>

namespace islbm {

namespace {

// Periodic-hill profile segments (C/model.h:17-53): value at distance t from the crest.
double segment(int s, double t) {
    switch (s) {
    case 1: return 1./28.*std::fmin(28., 28. + 0.006775070969851*t*28*t*28 - 0.0021245277758000*t*28*t*28*t*28);
    case 2: return 1./28.*(25.07355893131 + 0.9754803562315*t*28 - 0.1016116352781*t*28*t*28 + 0.001889794677828*t*28*t*28*t*28);
    case 3: return 1./28.*(25.79601052357 + 0.8206693007457*t*28 - 0.09055370274339*t*28*t*28 + 0.001626510569859*t*28*t*28*t*28);
    case 4: return 1./28.*(40.46435022819 - 1.379581654948*t*28 + 0.019458845041284*t*28*t*28 - 0.0002070318932190*t*28*t*28*t*28);
    case 5: return 1./28.*(17.92461334664 + 0.8743920332081*t*28 - 0.05567361123058*t*28*t*28 + 0.0006277731764683*t*28*t*28*t*28);
    default: return 1./28.*std::fmax(0., 56.39011190988 - 2.010520359035*t*28 + 0.01644919857549*t*28*t*28 + 0.00002674976141766*t*28*t*28*t*28);
    }
}

// Segment breakpoints in hill heights: (54/28)*(n/54), n = 9, 14, 20, 30, 40, 54.
const double kBreak[6] = {(54./28.)*(9./54.), (54./28.)*(14./54.), (54./28.)*(20./54.),
                          (54./28.)*(30./54.), (54./28.)*(40./54.), (54./28.)*(54./54.)};

double tanh_map(double L, double cell, double a, int j, int N) {
    return L/2.0 + cell/2.0 + ((L/2.0)/a)*std::tanh((-1.0 + 2.0*(double)(j)/(double)(N))/2.0*std::log((1.0 + a)/(1.0 - a)));
}

double lagrange6(double x, double xi, const double *others) {
    double r = (x - others[0])/(xi - others[0]);
    for (int m = 1; m < 6; m++) { r = r*(x - others[m]); r = r/(xi - others[m]); }
    return r;
}

// 7 weights of the Lagrange polynomial through nodes[n..n+6] at `pos`, stored with stride
// `stride` at `store` (C/initializationTool.h:68-79).
void weights7(double *dst, size_t stride, size_t store, double pos, const double *nodes, int n) {
    for (int a = 0; a < 7; a++) {
        double others[6];
        int c = 0;
        for (int b = 0; b < 7; b++) if (b != a) others[c++] = nodes[n + b];
        dst[(size_t)a*stride + store] = lagrange6(pos, nodes[n + a], others);
    }
}

}  // namespace

double Geometry::hill(double Y) const {
    if (channel) return 0.0;   // ChannelFunction, C/model.h:70-73
    double Yb = Y;
    if (Y < 0.0) Yb = Y + LY; else if (Y > LY) Yb = Y - LY;
    if (alpha != 1.0) {
        // steepness extension: footprint stretched by alpha, height kept
        const double t = (Yb <= 0.5*LY ? Yb : LY - Yb)/alpha;
        for (int m = 0; m < 6; m++) if (t <= kBreak[m]) return segment(m + 1, t);
        return 0.0;
    }
    double model = 0.0;
    if (Yb <= kBreak[0]) model = segment(1, Yb);
    if (Yb > kBreak[0] && Yb <= kBreak[1]) model = segment(2, Yb);
    if (Yb > kBreak[1] && Yb <= kBreak[2]) model = segment(3, Yb);
    if (Yb > kBreak[2] && Yb <= kBreak[3]) model = segment(4, Yb);
    if (Yb > kBreak[3] && Yb <= kBreak[4]) model = segment(5, Yb);
    if (Yb > kBreak[4] && Yb <= kBreak[5]) model = segment(6, Yb);
    const double t = LY - Yb;
    if (Yb < LY - kBreak[4] && Yb >= LY - kBreak[5]) model = segment(6, t);
    if (Yb < LY - kBreak[3] && Yb >= LY - kBreak[4]) model = segment(5, t);
    if (Yb < LY - kBreak[2] && Yb >= LY - kBreak[3]) model = segment(4, t);
    if (Yb < LY - kBreak[1] && Yb >= LY - kBreak[2]) model = segment(3, t);
    if (Yb < LY - kBreak[0] && Yb >= LY - kBreak[1]) model = segment(2, t);
    if (Yb >= LY - kBreak[0]) model = segment(1, t);
    return model;
}

int Geometry::cell_z(int k) const {
    int c = k - 3;
    if (k <= 6) c = 3;
    if (k >= NZ6 - 7) c = NZ6 - 10;
    return c;
}

int validate(const islbm_params &p) {
    if (p.NX < 1 || p.NY < 8 || p.NZ < 8) return ISLBM_ERR_INVALID_ARGUMENT;
    if ((long long)p.NX*p.NY*p.NZ > (1LL << 34)) return ISLBM_ERR_INVALID_ARGUMENT;
    if (!(p.LX > 0) || !(p.LY > 0) || !(p.LZ > 1.0) || !(p.CFL > 0) || !(p.LXi > 0)) return ISLBM_ERR_INVALID_ARGUMENT;
    if (!(p.Re > 0) || !(p.Uref > 0) || p.NDTFRC < 1) return ISLBM_ERR_INVALID_ARGUMENT;
    if (p.precision < ISLBM_FP64 || p.precision > ISLBM_BF16_DEV) return ISLBM_ERR_INVALID_ARGUMENT;
    if (p.les_cs < 0 || !(p.alpha > 0) || p.init_mode < 0 || p.init_mode > 1) return ISLBM_ERR_INVALID_ARGUMENT;
    if (p.mass_interval < 0 || p.bfl_mode < 0 || p.bfl_mode > 1) return ISLBM_ERR_INVALID_ARGUMENT;
    if (p.geometry < 0 || p.geometry > 1) return ISLBM_ERR_INVALID_ARGUMENT;
    if (p.kernel < ISLBM_KERNEL_AUTO || p.kernel > ISLBM_KERNEL_TILED_SINGLE) return ISLBM_ERR_INVALID_ARGUMENT;
    if (p.alpha != 1.0 && p.LY < 2.0*kBreak[5]*p.alpha) return ISLBM_ERR_INVALID_ARGUMENT;
    return ISLBM_OK;
}

int Geometry::build(const islbm_params &p) {
    const int st = validate(p);
    if (st != ISLBM_OK) return st;
    NX = p.NX; NY = p.NY; NZ = p.NZ;
    NX6 = NX + 7; NYD6 = NY + 7; NZ6 = NZ + 6;
    LX = p.LX; LY = p.LY; LZ = p.LZ; CFL = p.CFL; LXi = p.LXi; Re = p.Re; alpha = p.alpha; channel = p.geometry == 1;
    minSize = ((LZ - 1.0)/(double)(NZ6 - 6))*CFL;
    dt = minSize;
    tau = 0.5 + 3.0*(p.Uref)/((double)Re*minSize);
    niu = ((tau - 0.5)/3.0*dt);
    Uref = (Re*niu);
    force0 = (8.0*niu*Uref)/(LZ*LZ)*5.0;

    const size_t nyz = (size_t)NYD6*NZ6, nb = 2*(size_t)NYD6;
    x.assign(NX6, 0.0); y.assign(NYD6, 0.0); z.assign(nyz, 0.0); xi.assign(NZ6, 0.0);
    XP0.assign(7*(size_t)NX6, 0.0); XP2.assign(7*(size_t)NX6, 0.0);
    YP0.assign(7*(size_t)NYD6, 0.0); YP2.assign(7*(size_t)NYD6, 0.0);
    XiT.assign(8*7*nyz, 0.0);
    bfl.assign(4*nb, 0); Q.assign(4*nb, 0.0); BW.assign((size_t)NBFL*7*nb, 0.0);

    // GenerateMesh_X / _Y (uniform; jp = 1 so y_h = y_global)
    const double dx = LX/(double)(NX6 - 2*3 - 1);
    for (int i = 0; i < NX6; i++) x[i] = dx*((double)(i - 3));
    const double dy = LY/(double)((NY + 7) - 2*3 - 1);
    for (int j = 0; j < NYD6; j++) y[j] = dy*((double)(j - 3));

    // GetNonuniParameter: bisection for the tanh factor whose first spacing is minSize
    {
        const double total = LZ - hill(0.0) - minSize;
        double a0 = 0.1, a1 = 1.0, mid, d;
        int it = 0;
        do {
            mid = (a0 + a1)/2.0;
            d = tanh_map(total, minSize, mid, 1, NZ6 - 7) - tanh_map(total, minSize, mid, 0, NZ6 - 7);
            if (d - minSize >= 0.0) a0 = mid; else a1 = mid;
        } while (std::fabs(d - minSize) > 1e-14 && ++it < 400);
        a_nonuni = mid;
    }
    // GenerateMesh_Z: body-fitted tanh-stretched columns
    for (int j = 0; j < NYD6; j++) {
        const double total = LZ - hill(y[j]) - minSize;
        for (int k = 3; k < NZ6 - 3; k++) z[(size_t)j*NZ6 + k] = tanh_map(total, minSize, a_nonuni, k - 3, NZ6 - 7) + hill(y[j]);
        z[(size_t)j*NZ6 + 2] = hill(y[j]);
        z[(size_t)j*NZ6 + (NZ6 - 3)] = LZ;
    }
    for (int k = 3; k < NZ6 - 3; k++) xi[k] = tanh_map(LXi, minSize, a_nonuni, k - 3, NZ6 - 7) - minSize/2.0;

    // GetIntrplParameter_X / _Y
    for (int i = 3; i < NX6 - 3; i++) {
        weights7(XP0.data(), NX6, i, x[i] - minSize, x.data(), i - 3);
        weights7(XP2.data(), NX6, i, x[i] + minSize, x.data(), i - 3);
    }
    for (int j = 3; j < NYD6 - 3; j++) {
        weights7(YP0.data(), NYD6, j, y[j] - minSize, y.data(), j - 3);
        weights7(YP2.data(), NYD6, j, y[j] + minSize, y.data(), j - 3);
    }
    // GetXiParameter: weights in the xi coordinate at the departure point (pos_y, pos_z)
    auto xi_weights = [&](double *dst, size_t stride, size_t store, double pos_z, double pos_y, int k) {
        const double L = LZ - hill(pos_y) - minSize;
        const double pos_xi = LXi*(pos_z - (hill(pos_y) + minSize/2.0))/L;
        int base = k - 3;
        if (k >= 3 && k <= 6) base = 3;
        else if (k >= NZ6 - 7 && k <= NZ6 - 4) base = NZ6 - 10;
        weights7(dst, stride, store, pos_xi, xi.data(), base);
    };
    // GetIntrplParameter_Xi: departure points of F3,4,5,6,15,16,17,18
    const double dyz[8][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}, {-1, -1}, {1, -1}, {-1, 1}, {1, 1}};  // (dy, dz)/minSize
    for (int j = 3; j < NYD6 - 3; j++)
        for (int k = 3; k < NZ6 - 3; k++) {
            const double zz = z[(size_t)j*NZ6 + k], yy = y[j];
            for (int t = 0; t < 8; t++) {
                const double pz = dyz[t][1] == 0 ? zz : (dyz[t][1] < 0 ? zz - minSize : zz + minSize);
                const double py = dyz[t][0] == 0 ? yy : (dyz[t][0] < 0 ? yy - minSize : yy + minSize);
                xi_weights(&XiT[(size_t)t*7*nyz], nyz, (size_t)j*NZ6 + k, pz, py, k);
            }
        }

    // BFLInitialization: flags, wall distances Q and the weights of the Q < 0.5 branch
    for (int k = 0; k < 2; k++)
        for (int j = 3; j < NYD6 - 3; j++) {
            const size_t r = (size_t)k*NYD6 + j;
            const double zz = z[(size_t)j*NZ6 + k + 3];
            bfl[0*nb + r] = hill(y[j] - minSize) > zz ? 1 : 0;
            bfl[1*nb + r] = hill(y[j] + minSize) > zz ? 1 : 0;
            bfl[2*nb + r] = hill(y[j] - minSize) > zz - minSize ? 1 : 0;
            bfl[3*nb + r] = hill(y[j] + minSize) > zz - minSize ? 1 : 0;
        }
    auto delta_horizontal = [&](double z_target, double y_large, double y_small, double y_point) {
        double t0 = y_large, t1 = y_small, mid;
        int it = 0;
        do {
            mid = (t0 + t1)/2.0;
            if (hill(mid) >= z_target) t0 = mid; else t1 = mid;
        } while (std::fabs(hill(mid) - z_target) > 1e-13 && ++it < 400);
        return minSize - 2.0*std::fabs(y_point - mid);
    };
    auto delta_45 = [&](double z_pnt, double y_pnt, double y_zdom, double y_ydom) {
        double t0 = y_zdom, t1 = y_ydom, mid;
        int it = 0;
        do {
            mid = (t0 + t1)/2.0;
            if (std::fabs(hill(mid) - z_pnt) > std::fabs(mid - y_pnt)) t0 = mid; else t1 = mid;
        } while (std::fabs(std::fabs(hill(mid) - z_pnt) - std::fabs(mid - y_pnt)) > 1e-13 && ++it < 400);
        return minSize - 2.0*std::fabs(y_pnt - mid);
    };
    auto bw = [&](int s) { return &BW[(size_t)s*7*nb]; };
    const double xm = x[NX6/2];
    for (int k = 0; k < 2; k++)
        for (int j = 3; j < NYD6 - 3; j++) {
            const size_t r = (size_t)k*NYD6 + j;
            const double zz = z[(size_t)j*NZ6 + k + 3], yy = y[j];
            if (bfl[0*nb + r] == 1) {
                const double delta = delta_horizontal(zz, yy - minSize, yy, yy);
                Q[0*nb + r] = (minSize - delta)/2.0/minSize;
                weights7(bw(XB38), nb, r, xm - delta, x.data(), NX6/2 - 3);
                weights7(bw(XB37), nb, r, xm + delta, x.data(), NX6/2 - 3);
                weights7(bw(YB378), nb, r, yy + delta, y.data(), j - 3);
                xi_weights(bw(XiB378), nb, r, zz, yy + delta, k + 3);
            }
            if (bfl[1*nb + r] == 1) {
                const double delta = delta_horizontal(zz, yy + minSize, yy, yy);
                Q[1*nb + r] = (minSize - delta)/2.0/minSize;
                weights7(bw(XB49), nb, r, xm + delta, x.data(), NX6/2 - 3);
                weights7(bw(XB410), nb, r, xm - delta, x.data(), NX6/2 - 3);
                weights7(bw(YB4910), nb, r, yy - delta, y.data(), j - 3);
                xi_weights(bw(XiB4910), nb, r, zz, yy - delta, k + 3);
            }
            if (bfl[2*nb + r] == 1) {
                const double delta = delta_45(zz, yy, yy, yy - minSize);
                Q[2*nb + r] = (minSize - delta)/2.0/minSize;
                weights7(bw(YB15), nb, r, yy + delta, y.data(), j - 3);
                xi_weights(bw(XiB15), nb, r, zz + delta, yy + delta, k + 3);
            }
            if (bfl[3*nb + r] == 1) {
                const double delta = delta_45(zz, yy, yy, yy + minSize);
                Q[3*nb + r] = (minSize - delta)/2.0/minSize;
                weights7(bw(YB16), nb, r, yy - delta, y.data(), j - 3);
                xi_weights(bw(XiB16), nb, r, zz + delta, yy - delta, k + 3);
            }
        }
    return ISLBM_OK;
}

const double *Geometry::table(const std::string &name, int idx, size_t *count) const {
    const size_t nyz = (size_t)NYD6*NZ6, nb = 2*(size_t)NYD6;
    if (idx < 0 || idx > 6) idx = 0;
    static const char *xi_names[8] = {"XiF3", "XiF4", "XiF5", "XiF6", "XiF15", "XiF16", "XiF17", "XiF18"};
    static const char *bfl_names[NBFL] = {"XBFL37", "XBFL38", "YBFL378", "XiBFL378", "XBFL49", "XBFL410",
                                          "YBFL4910", "XiBFL4910", "YBFL15", "XiBFL15", "YBFL16", "XiBFL16"};
    static const char *q_names[4] = {"Q3", "Q4", "Q15", "Q16"};
    if (name == "x") { *count = x.size(); return x.data(); }
    if (name == "y") { *count = y.size(); return y.data(); }
    if (name == "z") { *count = z.size(); return z.data(); }
    if (name == "xi") { *count = xi.size(); return xi.data(); }
    if (name == "XPara0") { *count = NX6; return &XP0[(size_t)idx*NX6]; }
    if (name == "XPara2") { *count = NX6; return &XP2[(size_t)idx*NX6]; }
    if (name == "YPara0") { *count = NYD6; return &YP0[(size_t)idx*NYD6]; }
    if (name == "YPara2") { *count = NYD6; return &YP2[(size_t)idx*NYD6]; }
    for (int t = 0; t < 8; t++) if (name == xi_names[t]) { *count = nyz; return &XiT[((size_t)t*7 + idx)*nyz]; }
    for (int s = 0; s < NBFL; s++) if (name == bfl_names[s]) { *count = nb; return &BW[((size_t)s*7 + idx)*nb]; }
    for (int t = 0; t < 4; t++) if (name == q_names[t]) { *count = nb; return &Q[(size_t)t*nb]; }
    *count = 0;
    return nullptr;
}

const int *Geometry::table_int(const std::string &name, size_t *count) const {
    const size_t nb = 2*(size_t)NYD6;
    static const char *names[4] = {"BFL3", "BFL4", "BFL15", "BFL16"};
    for (int t = 0; t < 4; t++) if (name == names[t]) { *count = nb; return &bfl[(size_t)t*nb]; }
    *count = 0;
    return nullptr;
}

}  // namespace islbm
