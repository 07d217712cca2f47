// Point force fields on the host (see force_fields.h).  The arithmetic keeps
// the reference's float/double steps: positions from Grid3d's index maps
// (grid3d.h:77-125), vmath's float length and normalisation (vmath.h:86-97,
// vmath.cpp:81-110), and the FP64 trilinear interpolation of a nodal grid
// (interpolation.cpp:61-112).
#include "force_fields.h"

#include <algorithm>
#include <cmath>
#include <limits>

namespace flip {

namespace {

struct V3 {
    float x, y, z;
};
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 scale(float s, V3 v) { return {v.x * s, v.y * s, v.z * s}; }   // operator*(float, vec3)
inline float length(V3 v) { return std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }
// vmath::normalize: v / |v|, as v times the float of 1.0 / |v|
inline V3 normalize(V3 v) {
    const float inv = (float)(1.0 / (double)length(v));
    return {v.x * inv, v.y * inv, v.z * inv};
}
// Grid3d::GridIndexToPosition and FaceIndexToPositionU/V/W: FP64 products
// rounded to float
inline float at_node(int i, double dx) { return (float)((double)(float)i * dx); }
inline float at_centre(int i, double dx) { return (float)(((double)(float)i + 0.5) * dx); }
inline V3 face_position(int dir, int i, int j, int k, double dx) {
    return {dir == 0 ? at_node(i, dx) : at_centre(i, dx), dir == 1 ? at_node(j, dx) : at_centre(j, dx),
            dir == 2 ? at_node(k, dx) : at_centre(k, dx)};
}

// ForceField::_calculateForceVector and _limitForceVector (forcefield.cpp:
// 215-235): strength / r^falloff along the normal, its length capped at
// |strength| times the limit factor.
V3 force_vector(const PointForceField &f, float distance, V3 normal) {
    const float eps = 1e-6f;
    const float s = f.strength * (1.0f / powf(distance, f.falloffPower));
    V3 force = scale(s, normal);
    const float maxForce = std::abs(f.strength) * f.maxForceLimitFactor;
    const float len = length(force);
    if (len <= maxForce || len < eps) return force;
    if (maxForce < eps) return {0.f, 0.f, 0.f};
    return scale(maxForce / len, force);
}

// Interpolation::trilinearInterpolate(vec3 p, double dx, Array3d<float>)
// (interpolation.cpp:61-112) on a nodal grid of a x b x c values; indices
// outside it read zero.
double trilinear_nodal(V3 p, double dx, const std::vector<float> &g, int a, int b, int c) {
    const double invdx = 1.0 / dx;
    const int gi = (int)std::floor((double)p.x * invdx), gj = (int)std::floor((double)p.y * invdx),
              gk = (int)std::floor((double)p.z * invdx);
    const V3 gpos = {at_node(gi, dx), at_node(gj, dx), at_node(gk, dx)};
    const double ix = (double)(p.x - gpos.x) * invdx, iy = (double)(p.y - gpos.y) * invdx,
                 iz = (double)(p.z - gpos.z) * invdx;
    auto val = [&](int i, int j, int k) -> double {
        if (i < 0 || j < 0 || k < 0 || i >= a || j >= b || k >= c) return 0.0;
        return g[(size_t)i + (size_t)a * ((size_t)j + (size_t)b * k)];
    };
    const double p0 = val(gi, gj, gk), p1 = val(gi + 1, gj, gk), p2 = val(gi, gj + 1, gk),
                 p3 = val(gi, gj, gk + 1), p4 = val(gi + 1, gj, gk + 1), p5 = val(gi, gj + 1, gk + 1),
                 p6 = val(gi + 1, gj + 1, gk), p7 = val(gi + 1, gj + 1, gk + 1);
    const double x = ix, y = iy, z = iz;
    return p0 * (1 - x) * (1 - y) * (1 - z) + p1 * x * (1 - y) * (1 - z) + p2 * (1 - x) * y * (1 - z) +
           p3 * (1 - x) * (1 - y) * z + p4 * x * (1 - y) * z + p5 * (1 - x) * y * z + p6 * x * y * (1 - z) +
           p7 * x * y * z;
}

}  // namespace

void mesh_centroid(const float *verts, int nverts, float out[3]) {
    float c[3] = {0.f, 0.f, 0.f};
    for (int q = 0; q < nverts; q++)
        for (int d = 0; d < 3; d++) c[d] += verts[3 * q + d];
    if (nverts > 0) {
        const float inv = (float)(1.0 / (double)(float)nverts);   // vec3 /= (float)size
        for (int d = 0; d < 3; d++) c[d] *= inv;
    }
    for (int d = 0; d < 3; d++) out[d] = c[d];
}

void point_force_grid(int ni, int nj, int nk, double dx, const std::vector<PointForceField> &fields,
                      const float gravity[3], ForceFieldGridHost &out) {
    out.ni = ni;
    out.nj = nj;
    out.nk = nk;
    out.dx = dx;
    std::vector<float> *comp[3] = {&out.u, &out.v, &out.w};
    const int ext[3][3] = {{ni + 1, nj, nk}, {ni, nj + 1, nk}, {ni, nj, nk + 1}};
    for (int d = 0; d < 3; d++) comp[d]->assign((size_t)ext[d][0] * ext[d][1] * ext[d][2], 0.0f);
    const float eps = 1e-6f;

    // _applyForceFields: ForceFieldPoint::_addForceFieldToGridThread
    // (forcefieldpoint.cpp:146-217), U then V then W of each field in turn
    for (const PointForceField &f : fields) {
        if (!f.enabled) continue;
        const V3 p = {f.cx, f.cy, f.cz};
        const float minDistance = f.minDistanceEnabled ? f.minDistance : -1.0f;
        const float maxDistance = f.maxDistanceEnabled ? f.maxDistance : std::numeric_limits<float>::infinity();
        for (int d = 0; d < 3; d++) {
            const int a = ext[d][0], b = ext[d][1], c = ext[d][2];
            std::vector<float> &G = *comp[d];
            for (int k = 0; k < c; k++)
                for (int j = 0; j < b; j++)
                    for (int i = 0; i < a; i++) {
                        const V3 v = sub(face_position(d, i, j, k, dx), p);
                        const float r = std::max(length(v), minDistance);
                        if (r < eps || r > maxDistance) continue;
                        const V3 force = force_vector(f, r, normalize(v));
                        G[(size_t)i + (size_t)a * ((size_t)j + (size_t)b * k)] +=
                            d == 0 ? force.x : (d == 1 ? force.y : force.z);
                    }
        }
    }

    // _applyGravity (forcefieldgrid.cpp:263-313): the gravity-scale grid
    // (ForceFieldPoint::addGravityScaleToGrid, forcefieldpoint.cpp:53-73, and
    // ForceFieldGravityScaleGrid::normalize), then gravity times the scale
    // interpolated at each face
    const int na = ni + 1, nb = nj + 1, nc = nk + 1;
    std::vector<float> sum((size_t)na * nb * nc, 0.0f);
    std::vector<int> count(sum.size(), 0);
    for (const PointForceField &f : fields) {
        if (!f.enabled) continue;
        float width = f.gravityScaleWidth;
        if (f.maxDistanceEnabled) width = std::min(width, f.maxDistance);
        const V3 p = {f.cx, f.cy, f.cz};
        for (int k = 0; k < nc; k++)
            for (int j = 0; j < nb; j++)
                for (int i = 0; i < na; i++) {
                    const float dist = length(sub({at_node(i, dx), at_node(j, dx), at_node(k, dx)}, p));
                    if (dist < width) {
                        const float factor = 1.0f - (dist / width);
                        const float s = factor * f.gravityScale + (1.0f - factor);
                        const size_t e = (size_t)i + (size_t)na * ((size_t)j + (size_t)nb * k);
                        sum[e] += s;
                        count[e] += 1;
                    }
                }
    }
    for (size_t e = 0; e < sum.size(); e++) sum[e] = count[e] == 0 ? 1.0f : sum[e] / (float)count[e];
    for (int d = 0; d < 3; d++) {
        if (!(std::abs(gravity[d]) > eps)) continue;
        const int a = ext[d][0], b = ext[d][1], c = ext[d][2];
        std::vector<float> &G = *comp[d];
        for (int k = 0; k < c; k++)
            for (int j = 0; j < b; j++)
                for (int i = 0; i < a; i++) {
                    const float s = (float)trilinear_nodal(face_position(d, i, j, k, dx), dx, sum, na, nb, nc);
                    G[(size_t)i + (size_t)a * ((size_t)j + (size_t)b * k)] += s * gravity[d];
                }
    }
}

}  // namespace flip
