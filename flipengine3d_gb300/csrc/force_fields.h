// Force fields on the host: the point fields of ForceFieldGrid
// (forcefieldgrid.cpp, forcefieldpoint.cpp, forcefield.cpp).  The grid is a
// MAC field on the (possibly reduced) force-field grid; it is rebuilt only
// when a field or the gravity vector changes, so it is set up here and
// uploaded, and the device applies it to the velocity faces every substep.
#pragma once

#include <vector>

namespace flip {

// One point field: the centroid of a static mesh and ForceField's parameters
// (forcefield.h:107-118 holds the defaults).
struct PointForceField {
    float cx = 0.f, cy = 0.f, cz = 0.f;   // TriangleMesh::getCentroid of the field's mesh
    float strength = 0.f;
    float falloffPower = 1.f;
    float maxForceLimitFactor = 3.f;
    bool minDistanceEnabled = false;
    float minDistance = 0.f;
    bool maxDistanceEnabled = false;
    float maxDistance = 0.f;
    float gravityScale = 1.f;
    float gravityScaleWidth = 0.f;
    bool enabled = true;
};

// The force-field grid: faces of an ni x nj x nk grid of cell size dx.
struct ForceFieldGridHost {
    int ni = 0, nj = 0, nk = 0;
    double dx = 0.0;
    std::vector<float> u, v, w;   // (ni+1) nj nk, ni (nj+1) nk, ni nj (nk+1)
};

// TriangleMesh::getCentroid (trianglemesh.cpp:523-534): the float sum of the
// vertices times the float reciprocal of their count.
void mesh_centroid(const float *verts, int nverts, float out[3]);

// ForceFieldGrid::update (forcefieldgrid.cpp:73-95) from a cleared field:
// every enabled field's forces (_applyForceFields), then gravity scaled by
// the fields' gravity-scale grid (_applyGravity).
void point_force_grid(int ni, int nj, int nk, double dx, const std::vector<PointForceField> &fields,
                      const float gravity[3], ForceFieldGridHost &out);

}  // namespace flip
