// Result files of the reference, written from a solve's current fields.
//
//   islbm_write_tecplot_ascii  fileIO_velocity (C/fileIO.h:69-87): Tecplot POINT zone with X, Y, Z,
//                              U, V, W on the (NX+1) x (NY+1) x NZ nodes i, j, k = 3 .. N6-4 of
//                              the padded layout (the periodic end nodes included), coordinates
//                              with 4 decimals and velocities with 15;
//   islbm_write_tecplot_plt    Output3Dvelocity (C/fileIO.h:502-659): the same nodes in Tecplot's
//                              binary format #!TDV101, double precision, velocities / Uref;
//   islbm_write_monitor        Launch_Monitor (C/monitor.h:4-26): appends "step v u w force" for
//                              the node (NX6/2, NYD6/2, NZ6/2) to a text file.
// Coordinates are the mesh of the solve (x_h, y_h, z_h of C/initialization.h:51-183).
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "handle.hpp"

namespace {

struct Fields {
    int NX6, NYD6, NZ6;
    std::vector<double> u, v, w;
};

int fetch(islbm_handle *h, Fields &f) {
    f.NX6 = h->p.NX + 7; f.NYD6 = h->p.NY + 7; f.NZ6 = h->p.NZ + 6;
    const size_t n = (size_t)f.NX6*f.NYD6*f.NZ6;
    f.u.resize(n); f.v.resize(n); f.w.resize(n);
    return islbm_fields(h, nullptr, f.u.data(), f.v.data(), f.w.data(), ISLBM_LAYOUT_REFERENCE);
}

// Tecplot binary string: one 32-bit integer per character, then a zero
void put_str(FILE *fp, const char *s) {
    for (; *s; ++s) {
        const int c = (unsigned char)*s;
        std::fwrite(&c, sizeof(int), 1, fp);
    }
    const int z = 0;
    std::fwrite(&z, sizeof(int), 1, fp);
}
void put_i(FILE *fp, int v) { std::fwrite(&v, sizeof(int), 1, fp); }
void put_f(FILE *fp, float v) { std::fwrite(&v, sizeof(float), 1, fp); }
void put_d(FILE *fp, double v) { std::fwrite(&v, sizeof(double), 1, fp); }

int open_fail(const char *path) {
    return islbm::report_status(ISLBM_ERR_INVALID_ARGUMENT, (std::string("cannot write ") + path).c_str());
}

}  // namespace

extern "C" {

int islbm_write_tecplot_ascii(islbm_handle *h, const char *path) {
    if (!h || !path) return ISLBM_ERR_INVALID_ARGUMENT;
    Fields f;
    const int st = fetch(h, f);
    if (st != ISLBM_OK) return st;
    FILE *fp = std::fopen(path, "w");
    if (!fp) return open_fail(path);
    const auto &g = h->g;
    std::fprintf(fp, "VARIABLES = \"X\", \"Y\", \"Z\", \"U\", \"V\", \"W\"\n");
    std::fprintf(fp, "ZONE T = \"velocity\", F = POINT\n");
    std::fprintf(fp, "I = %d, J = %d, K = %d\n", f.NX6 - 6, f.NYD6 - 6, f.NZ6 - 6);
    for (int k = 3; k < f.NZ6 - 3; k++)
        for (int j = 3; j < f.NYD6 - 3; j++)
            for (int i = 3; i < f.NX6 - 3; i++) {
                const size_t idx = (size_t)j*f.NZ6*f.NX6 + (size_t)k*f.NX6 + i;
                std::fprintf(fp, "%.4lf\t %.4lf\t %.4lf\t ", g.x[i], g.y[j], g.z[(size_t)j*f.NZ6 + k]);
                std::fprintf(fp, "%.15lf\t %.15lf\t %.15lf\n", f.u[idx], f.v[idx], f.w[idx]);
            }
    if (std::fclose(fp) != 0) return open_fail(path);
    return ISLBM_OK;
}

int islbm_write_tecplot_plt(islbm_handle *h, const char *path) {
    if (!h || !path) return ISLBM_ERR_INVALID_ARGUMENT;
    Fields f;
    const int st = fetch(h, f);
    if (st != ISLBM_OK) return st;
    FILE *fp = std::fopen(path, "wb");
    if (!fp) return open_fail(path);
    const auto &g = h->g;
    const float zone_marker = 299.0f, eoh_marker = 357.0f;
    // header: magic, byte order, title, variables, one ordered zone of (I, J, K) points
    std::fwrite("#!TDV101", 8, 1, fp);
    put_i(fp, 1);
    put_str(fp, "Particle intensity");
    put_i(fp, 6);
    for (const char *name : {"X", "Y", "Z", "U", "V", "W"}) put_str(fp, name);
    put_f(fp, zone_marker);
    put_str(fp, "Zone 001");
    put_i(fp, -1);   // zone colour
    put_i(fp, 0);    // ordered zone
    put_i(fp, 1);    // point packing
    put_i(fp, 0);    // values at the nodes
    put_i(fp, 0);    // no face neighbour connections
    put_i(fp, f.NX6 - 6); put_i(fp, f.NYD6 - 6); put_i(fp, f.NZ6 - 6);
    put_i(fp, 0);    // no auxiliary name/value pairs
    put_f(fp, eoh_marker);
    // data: zone marker, six double variables, no sharing, then the points
    put_f(fp, zone_marker);
    for (int v = 0; v < 6; v++) put_i(fp, 2);
    put_i(fp, 0);
    put_i(fp, -1);
    const double uref = g.Uref;
    for (int k = 3; k < f.NZ6 - 3; k++)
        for (int j = 3; j < f.NYD6 - 3; j++)
            for (int i = 3; i < f.NX6 - 3; i++) {
                const size_t idx = (size_t)j*f.NZ6*f.NX6 + (size_t)k*f.NX6 + i;
                put_d(fp, g.x[i]); put_d(fp, g.y[j]); put_d(fp, g.z[(size_t)j*f.NZ6 + k]);
                put_d(fp, f.u[idx]/uref); put_d(fp, f.v[idx]/uref); put_d(fp, f.w[idx]/uref);
            }
    if (std::fclose(fp) != 0) return open_fail(path);
    return ISLBM_OK;
}

int islbm_write_monitor(islbm_handle *h, const char *path, int step) {
    if (!h || !path) return ISLBM_ERR_INVALID_ARGUMENT;
    Fields f;
    int st = fetch(h, f);
    if (st != ISLBM_OK) return st;
    double force = 0.0;
    st = islbm_get_scalars(h, &force, nullptr, nullptr);
    if (st != ISLBM_OK) return st;
    const int i = f.NX6/2, j = f.NYD6/2, k = f.NZ6/2;
    const size_t idx = (size_t)j*f.NX6*f.NZ6 + (size_t)k*f.NX6 + i;
    FILE *fp = std::fopen(path, "a");
    if (!fp) return open_fail(path);
    std::fprintf(fp, "%d\t %.15lf\t %.15lf\t %.15lf\t %.15lf\n", step, f.v[idx], f.u[idx], f.w[idx], force);
    if (std::fclose(fp) != 0) return open_fail(path);
    return ISLBM_OK;
}

}  // extern "C"
