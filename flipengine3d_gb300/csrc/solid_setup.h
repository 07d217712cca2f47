// Static solid set-up: the domain walls and static mesh obstacles (host,
// once per solid configuration).
#pragma once
#include <cstdint>
#include <vector>

namespace flip {

// A static triangle-mesh obstacle (addMeshObstacle, fluidsimulation.cpp:
// 1994-2008): world-space vertices, triangles as vertex index triples, and
// the friction its faces apply in the constrain step (MeshObject::setFriction,
// meshobject.cpp:301-309).
struct MeshObstacle {
    std::vector<float> verts;   // x, y, z per vertex
    std::vector<int> tris;      // three vertex indices per triangle
    float friction = 0.0f;
};

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
    // per node: the solid object closest to it (-1 none, 0 the domain walls,
    // q + 1 obstacle q) and that object's friction; per face the mean friction
    // of its four nodes (fluidsimulation.cpp:3785-3846)
    std::vector<int> nodeObject;
    std::vector<float> nodeFriction;
    std::vector<float> fu, fv, fw;
    bool anyFriction = false;

    void compute(int I, int J, int K, double dx, double cfl, const std::vector<MeshObstacle> &obstacles = {});
};

// A fluid mesh's seeding inputs (addMeshFluid): the cells of the grid nodes
// inside the mesh, ascending flat index, and its (I+1)(J+1)(K+1) nodal level
// set, negative inside.
void mesh_fluid_cells(int I, int J, int K, double dx, const std::vector<float> &verts, const std::vector<int> &tris,
                      std::vector<int> &cells, std::vector<float> &phi);

// The host set-up of a static mesh fluid source (MeshFluidSource::update,
// meshfluidsource.cpp:171-214, 300-318): the cells of the grid nodes inside
// the mesh (MeshObject::getCells), and the mesh's level set over the
// sub-grid its bounding box spans, padded by 4 cells and clamped to the
// domain, exact in a band of 2, with its first node at `offset`.
struct SourceGrid {
    int gmin[3] = {0, 0, 0};     // first cell of the sub-grid
    int nodes[3] = {1, 1, 1};    // nodes of the level set (cells + 1)
    float offset[3] = {0, 0, 0}; // position of its first node
    std::vector<float> phi;      // negative inside
    std::vector<int> cells;      // flat indices, ascending
};
void fluid_source_setup(int I, int J, int K, double dx, const std::vector<float> &verts, const std::vector<int> &tris,
                        SourceGrid &g);

}  // namespace flip
