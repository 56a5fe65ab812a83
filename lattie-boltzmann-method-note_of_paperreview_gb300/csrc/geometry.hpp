// Host FP64 precompute of the periodic-hill mesh, interpolation weights and BFL tables.
//
// Follows the reference's one-time setup (C/ = 筆記：金的code/0.可更改的code/):
//   HillFunction                      C/model.h:4-68
//   tanhFunction, GetNonuniParameter  C/initializationTool.h:4-39
//   Lagrange_6th, GetParameter_6th    C/initializationTool.h:60-79
//   IsBFLBCNeeded, GetDeltaHorizontal,
//   GetDelta45Degree                  C/initializationTool.h:81-154
//   GenerateMesh_X/Y/Z, GetXiParameter,
//   GetIntrplParameter_X/Y/Xi,
//   BFLInitialization                 C/initialization.h:51-360
// in the same operation order, so the tables equal the reference's bit for bit. Tables are
// kept in the reference's index space (i in [0,NX6), j in [0,NYD6), k in [0,NZ6), BFL rows
// r = (k-3)*NYD6 + j); the device packer cuts the unique nodes out of them.
#pragma once

#include <cstddef>
#include <string>
#include <vector>

#include "../../include/islbm.h"

namespace islbm {

struct Geometry {
    // grid (C/variables.h:10-19 with jp = 1)
    int NX = 0, NY = 0, NZ = 0, NX6 = 0, NYD6 = 0, NZ6 = 0;
    double LX = 0, LY = 0, LZ = 0, CFL = 0, LXi = 0, Re = 0, alpha = 1.0;
    bool channel = false;   // flat channel: ChannelFunction (C/model.h:70-73) instead of the hill
    // derived constants (C/variables.h:22, 76, 97-101)
    double minSize = 0, dt = 0, tau = 0, niu = 0, Uref = 0, a_nonuni = 0;
    double force0 = 0;  // C/initialization.h:46
    std::vector<double> x, y, z, xi;
    std::vector<double> XP0, XP2, YP0, YP2;   // [a*NX6 + i], [a*NYD6 + j]
    std::vector<double> XiT;                  // [(t*7 + a)*NYD6*NZ6 + j*NZ6 + k], t: F3,4,5,6,15,16,17,18
    std::vector<int> bfl;                     // [t*2*NYD6 + r], t: F3, F4, F15, F16
    std::vector<double> Q;                    // [t*2*NYD6 + r]
    std::vector<double> BW;                   // [(s*7 + a)*2*NYD6 + r], s in BflSet order

    enum BflSet { XB37 = 0, XB38, YB378, XiB378, XB49, XB410, YB4910, XiB4910, YB15, XiB15, YB16, XiB16, NBFL };

    int build(const islbm_params &p);   // returns islbm_status
    double hill(double Y) const;
    int cell_z(int k) const;            // stencil base in k (C/evolution.h:421-423)

    const double *table(const std::string &name, int idx, size_t *count) const;
    const int *table_int(const std::string &name, size_t *count) const;
};

int validate(const islbm_params &p);

}  // namespace islbm
