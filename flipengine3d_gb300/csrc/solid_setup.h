// Static solid set-up for the domain walls (host, once per simulation).
#pragma once
#include <cstdint>
#include <vector>

namespace flip {

struct DomainBox {
    int I = 0, J = 0, K = 0;
    double dx = 0;
    // boundary box (position float, extents double, as the reference's AABB)
    float px = 0, py = 0, pz = 0;
    double ex = 0, ey = 0, ez = 0;
    std::vector<float> nodal;              // (I+1)(J+1)(K+1) solid SDF, positive in the fluid region
    std::vector<float> wu, wv, ww;         // fluid face weights
    std::vector<uint8_t> solidCentre;      // I*J*K: solid SDF at the cell centre < 0
    std::vector<uint8_t> near;             // coarse near-solid grid
    int nsi = 0, nsj = 0, nsk = 0;
    double nearCell = 0;

    void compute(int I, int J, int K, double dx, double cfl);
};

}  // namespace flip
