// Static solid set-up for the domain walls (host, once per simulation).
//
// The reference builds its solid level set from the domain box mesh: the
// AABB (0,0,0)-(I dx, J dx, K dx) shrunk by 3 dx + 1e-4
// (fluidsimulation.cpp:2834-2839) as 12 triangles (:2806-2832), exact
// distances in a band of 3 nodes around each triangle, computed in the
// frame of the 10^3-node block holding the node (meshlevelset.cpp:878-918,
// 1114-1158), signs from inside/outside, then negated (:2927-2935).  Nodes
// outside every band keep the upper bound (I+J+K+3) dx.  From it: the face
// weights 1 - fractionInside(corners) (fluidsimulation.cpp:3690-3730), the
// "solid at cell centre" flags the liquid SDF post-process uses
// (particlelevelset.cpp:172-196, meshlevelset.cpp:152-162), and the coarse
// near-solid grid of the collision test (fluidsimulation.cpp:3083-3126).
// The walls are static, so this runs once; the per-step work is on the GPU.
#include "solid_setup.h"

#include <algorithm>
#include <cmath>

namespace flip {

namespace {

struct V { float x, y, z; };
inline V vsub(V a, V b) { return V{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V vadd(V a, V b) { return V{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V vscale(float s, V a) { return V{a.x * s, a.y * s, a.z * s}; }
inline float vdot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float vlen(V a) { return std::sqrt(vdot(a, a)); }
inline float gpos(int i, double dx) { return (float)((double)(float)i * dx); }

// Closest point of a (non-degenerate) triangle to p: Eberly's region
// classification on the parametric plane (s, t), with float edge vectors,
// FP64 region arithmetic and a float result point.
V closest_point(V p, V v0, V v1, V v2) {
    V e0 = vsub(v1, v0), e1 = vsub(v2, v0), d0 = vsub(v0, p);
    double a = vdot(e0, e0), b = vdot(e0, e1), c = vdot(e1, e1);
    double d = vdot(e0, d0), e = vdot(e1, d0);
    double det = a * c - b * b;
    double s = b * e - c * d, t = b * d - a * e;
    auto cl = [](double x) { return std::max(0.0, std::min(x, 1.0)); };
    if (s + t < det) {
        if (s < 0.0) {
            if (t < 0.0) {
                if (d < 0.0) { s = cl(-d / a); t = 0.0; }
                else { s = 0.0; t = cl(-e / c); }
            } else { s = 0.0; t = cl(-e / c); }
        } else if (t < 0.0) {
            s = cl(-d / a); t = 0.0;
        } else {
            double inv = 1.0 / det;
            s *= inv; t *= inv;
        }
    } else {
        double den = a - 2 * b + c;
        if (s < 0.0) {
            double t0 = b + d, t1 = c + e;
            if (t1 > t0) { s = cl((t1 - t0) / den); t = 1 - s; }
            else { t = cl(-e / c); s = 0.0; }
        } else if (t < 0.0) {
            if (a + d > b + e) { s = cl((c + e - b - d) / den); t = 1 - s; }
            else { s = cl(-e / c); t = 0.0; }
        } else {
            s = cl((c + e - b - d) / den); t = 1.0 - s;
        }
    }
    return vadd(vadd(v0, vscale((float)s, e0)), vscale((float)t, e1));
}

float frac2(float l, float r) {
    if (l < 0 && r < 0) return 1;
    if (l < 0 && r >= 0) return l / (l - r);
    if (l >= 0 && r < 0) return r / (r - l);
    return 0;
}

// Fraction of a square face inside the solid from its four corner values
// (marching squares on the corners, as LevelsetUtils::fractionInside does).
float frac4(float bl, float br, float tl, float tr) {
    int in = (bl < 0) + (tl < 0) + (br < 0) + (tr < 0);
    float q[4] = {bl, br, tr, tl};
    auto rot = [&q]() { float t = q[0]; q[0] = q[1]; q[1] = q[2]; q[2] = q[3]; q[3] = t; };
    if (in == 4) return 1;
    if (in == 0) return 0;
    if (in == 3) {
        while (q[0] < 0) rot();
        float a = 1 - frac2(q[0], q[3]), b = 1 - frac2(q[0], q[1]);
        return 1.0f - 0.5f * a * b;
    }
    if (in == 1) {
        while (q[0] >= 0) rot();
        float a = frac2(q[0], q[3]), b = frac2(q[0], q[1]);
        return 0.5f * a * b;
    }
    while (q[0] >= 0 || !(q[1] < 0 || q[2] < 0)) rot();
    if (q[1] < 0) return 0.5f * (frac2(q[0], q[3]) + frac2(q[1], q[2]));
    float mid = 0.25f * (q[0] + q[1] + q[2] + q[3]);
    if (mid < 0) {
        float area = 0;
        area += 0.5f * (1 - frac2(q[0], q[3])) * (1 - frac2(q[2], q[3]));
        area += 0.5f * (1 - frac2(q[0], q[1])) * (1 - frac2(q[2], q[1]));
        return 1.0f - area;
    }
    float area = 0;
    area += 0.5f * frac2(q[0], q[1]) * frac2(q[0], q[3]);
    area += 0.5f * frac2(q[2], q[1]) * frac2(q[2], q[3]);
    return area;
}

}  // namespace

void DomainBox::compute(int I_, int J_, int K_, double dx_, double cfl) {
    I = I_; J = J_; K = K_; dx = dx_;
    // boundary box: AABB::expand(-3dx - 1e-4): position -= h, extent += v
    double v = -3 * dx - 1e-4, h = 0.5 * v;
    px = 0.0f - (float)h; py = 0.0f - (float)h; pz = 0.0f - (float)h;
    ex = I * dx + v; ey = J * dx + v; ez = K * dx + v;
    const int ni = I + 1, nj = J + 1, nk = K + 1;
    nodal.assign((size_t)ni * nj * nk, (float)((double)(ni + nj + nk) * dx));
    auto nidx = [&](int i, int j, int k) { return (size_t)i + (size_t)ni * ((size_t)j + (size_t)nj * k); };
    float X1 = (float)(px + ex), Y1 = (float)(py + ey), Z1 = (float)(pz + ez);
    V c[8] = {{px, py, pz}, {X1, py, pz}, {X1, py, Z1}, {px, py, Z1}, {px, Y1, pz}, {X1, Y1, pz}, {X1, Y1, Z1}, {px, Y1, Z1}};
    const int tri[12][3] = {{0, 1, 2}, {0, 2, 3}, {4, 7, 6}, {4, 6, 5}, {0, 3, 7}, {0, 7, 4},
                            {1, 5, 6}, {1, 6, 2}, {0, 4, 5}, {0, 5, 1}, {3, 2, 6}, {3, 6, 7}};
    const int band = 3, bw = 10;
    for (int t = 0; t < 12; t++) {
        V a = c[tri[t][0]], b = c[tri[t][1]], e = c[tri[t][2]];
        float mn[3] = {std::min(a.x, std::min(b.x, e.x)), std::min(a.y, std::min(b.y, e.y)), std::min(a.z, std::min(b.z, e.z))};
        float mx[3] = {std::max(a.x, std::max(b.x, e.x)), std::max(a.y, std::max(b.y, e.y)), std::max(a.z, std::max(b.z, e.z))};
        int lo[3], hi[3], n[3] = {ni, nj, nk};
        for (int q = 0; q < 3; q++) {
            lo[q] = std::max(0, (int)std::floor(mn[q] * (1.0 / dx)) - band);
            hi[q] = std::min(n[q] - 1, (int)std::floor(mx[q] * (1.0 / dx)) + band + 1);
        }
        for (int k = lo[2]; k <= hi[2]; k++)
            for (int j = lo[1]; j <= hi[1]; j++)
                for (int i = lo[0]; i <= hi[0]; i++) {
                    V off{gpos(i / bw, (double)bw * dx), gpos(j / bw, (double)bw * dx), gpos(k / bw, (double)bw * dx)};
                    V g{gpos(i % bw, dx), gpos(j % bw, dx), gpos(k % bw, dx)};
                    float dist = vlen(vsub(closest_point(g, vsub(a, off), vsub(b, off), vsub(e, off)), g));
                    float &cur = nodal[nidx(i, j, k)];
                    if (dist < cur) cur = dist;
                }
    }
    // inside the box -> negative, then negate: the fluid region is positive
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++) {
                float gx = gpos(i, dx), gy = gpos(j, dx), gz = gpos(k, dx);
                bool inside = gx > px && gy > py && gz > pz && gx < px + ex && gy < py + ey && gz < pz + ez;
                float &val = nodal[nidx(i, j, k)];
                val = inside ? val : -val;
            }

    wu.assign((size_t)(I + 1) * J * K, 0.0f);
    wv.assign((size_t)I * (J + 1) * K, 0.0f);
    ww.assign((size_t)I * J * (K + 1), 0.0f);
    auto S = [&](int i, int j, int k) { return nodal[nidx(i, j, k)]; };
    auto wclamp = [](float f) { return std::max(0.0f, std::min(1.0f - f, 1.0f)); };
    for (int k = 0; k < K; k++)
        for (int j = 0; j < J; j++)
            for (int i = 0; i <= I; i++)
                wu[(size_t)i + (size_t)(I + 1) * ((size_t)j + (size_t)J * k)] =
                    wclamp(frac4(S(i, j, k), S(i, j + 1, k), S(i, j, k + 1), S(i, j + 1, k + 1)));
    for (int k = 0; k < K; k++)
        for (int j = 0; j <= J; j++)
            for (int i = 0; i < I; i++)
                wv[(size_t)i + (size_t)I * ((size_t)j + (size_t)(J + 1) * k)] =
                    wclamp(frac4(S(i, j, k), S(i, j, k + 1), S(i + 1, j, k), S(i + 1, j, k + 1)));
    for (int k = 0; k <= K; k++)
        for (int j = 0; j < J; j++)
            for (int i = 0; i < I; i++)
                ww[(size_t)i + (size_t)I * ((size_t)j + (size_t)J * k)] =
                    wclamp(frac4(S(i, j, k), S(i, j + 1, k), S(i + 1, j, k), S(i + 1, j + 1, k)));

    solidCentre.assign((size_t)I * J * K, 0);
    for (int k = 0; k < K; k++)
        for (int j = 0; j < J; j++)
            for (int i = 0; i < I; i++) {
                float cc = 0.125f * (S(i, j, k) + S(i + 1, j, k) + S(i, j + 1, k) + S(i + 1, j + 1, k) + S(i, j, k + 1) +
                                     S(i + 1, j, k + 1) + S(i, j + 1, k + 1) + S(i + 1, j + 1, k + 1));
                solidCentre[(size_t)i + (size_t)I * ((size_t)j + (size_t)J * k)] = cc < 0 ? 1 : 0;
            }

    // coarse near-solid grid: cells of 3 dx holding a node with |phi| < 3 dx,
    // dilated ceil(cfl / 3) times in the 6-neighbourhood
    const int nf = 3;
    nearCell = nf * dx;
    nsi = (int)std::ceil(I * dx / nearCell);
    nsj = (int)std::ceil(J * dx / nearCell);
    nsk = (int)std::ceil(K * dx / nearCell);
    near.assign((size_t)nsi * nsj * nsk, 0);
    auto cidx = [&](int i, int j, int k) { return (size_t)i + (size_t)nsi * ((size_t)j + (size_t)nsj * k); };
    float maxd = (float)(band * dx);
    for (int k = 0; k < K; k++)
        for (int j = 0; j < J; j++)
            for (int i = 0; i < I; i++)
                if (std::abs(S(i, j, k)) < maxd) near[cidx(i / nf, j / nf, k / nf)] = 1;
    int layers = (int)std::ceil((float)cfl / (float)nf);
    for (int l = 0; l < layers; l++) {
        std::vector<uint8_t> src = near;
        for (int k = 0; k < nsk; k++)
            for (int j = 0; j < nsj; j++)
                for (int i = 0; i < nsi; i++) {
                    if (!src[cidx(i, j, k)]) continue;
                    const int nb[6][3] = {{i - 1, j, k}, {i + 1, j, k}, {i, j - 1, k}, {i, j + 1, k}, {i, j, k - 1}, {i, j, k + 1}};
                    for (auto &q : nb)
                        if (q[0] >= 0 && q[1] >= 0 && q[2] >= 0 && q[0] < nsi && q[1] < nsj && q[2] < nsk)
                            near[cidx(q[0], q[1], q[2])] = 1;
                }
    }
}

}  // namespace flip
