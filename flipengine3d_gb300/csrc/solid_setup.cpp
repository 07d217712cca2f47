// Static solid set-up: the domain walls and static mesh obstacles (host,
// once per solid configuration).
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
// Each static mesh obstacle adds a level set over the sub-grid that its
// bounding box spans (meshobject.cpp:239-265, 515-553): the exact band in
// the same block frame, signs from the parity of z-ray crossings through the
// nodes (meshutils.cpp:99-215, 347-428), unioned into the walls' level set
// through a temporary one (fluidsimulation.cpp:2927-2966, meshlevelset.cpp:
// 603-638, 1758-1790).  The union also records, per node, which object is
// closest: its friction blends the velocity of part-solid faces in the
// constrain step (fluidsimulation.cpp:3785-3846, 3884-3935).
// The solids are static, so this runs once; the per-step work is on the GPU.
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

inline V cross(V a, V b) {
    return V{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline int floor_index(float p, double dx) { return (int)std::floor((double)p * (1.0 / dx)); }

// Collision::lineIntersectsTriangle (collision.cpp:79-118) for the ray
// direction (0, 0, 1), in its float arithmetic: the z of the crossing.
bool ray_z_crossing(V p, V v0, V v1, V v2, float *z) {
    const V dir{0.0f, 0.0f, 1.0f};
    const V e1 = vsub(v1, v0), e2 = vsub(v2, v0);
    const V h = cross(dir, e2);
    const float a = vdot(e1, h);
    if (std::fabs(a) < 10e-9) return false;
    const float f = 1 / a;
    const V s = vsub(p, v0);
    const float u = f * vdot(s, h);
    if (u < 0.0 || u > 1.0) return false;
    const V q = cross(s, e1);
    const float v = f * vdot(dir, q);
    if (v < 0.0 || u + v > 1.0) return false;
    const double t = f * vdot(e2, q);
    *z = p.z + (float)t * dir.z;
    return true;
}

// MeshUtils::getGridNodesInsideTriangleMesh for one mesh (meshutils.cpp:
// 347-371, 156-215): the nodes become the cell centres of a grid shifted by
// half a cell, and a node is inside when the z-ray through it crosses the
// mesh an even number of times in all and an odd number of times below it.
// `mark(i, j, k)` is called for each inside node (any index; the caller
// keeps those in range).  The reference jitters the ray origins by a random
// amount below 0.001 dx against rays that graze an edge; here the jitter is
// a fixed amount in that range.
template <class Mark>
void inside_nodes_of(const std::vector<V> &vtx, const std::vector<int> &tris, double dx, Mark &&mark) {
    const int ntri = (int)tris.size() / 3;
    const float half = (float)(0.5 * dx);
    std::vector<V> m(vtx.size());
    for (size_t q = 0; q < vtx.size(); q++) m[q] = vadd(vtx[q], V{half, half, half});
    if (m.empty() || ntri == 0) return;
    float bmin[3] = {m[0].x, m[0].y, m[0].z}, bmax[3] = {m[0].x, m[0].y, m[0].z};
    for (const V &v : m) {
        bmin[0] = std::min(bmin[0], v.x); bmin[1] = std::min(bmin[1], v.y); bmin[2] = std::min(bmin[2], v.z);
        bmax[0] = std::max(bmax[0], v.x); bmax[1] = std::max(bmax[1], v.y); bmax[2] = std::max(bmax[2], v.z);
    }
    const double bext[3] = {(double)bmax[0] - bmin[0], (double)bmax[1] - bmin[1], (double)bmax[2] - bmin[2]};
    const int go[3] = {floor_index(bmin[0], dx), floor_index(bmin[1], dx), floor_index(bmin[2], dx)};
    const V offset{gpos(go[0], dx), gpos(go[1], dx), gpos(go[2], dx)};
    const V noff{-offset.x, -offset.y, -offset.z};
    for (V &v : m) v = vadd(v, noff);
    float bpos[3] = {bmin[0] - offset.x, bmin[1] - offset.y, bmin[2] - offset.z};
    const int cI = floor_index(bpos[0] + (float)bext[0], dx) + 1;
    const int cJ = floor_index(bpos[1] + (float)bext[1], dx) + 1;
    const int cK = floor_index(bpos[2] + (float)bext[2], dx) + 1;
    if (cI <= 0 || cJ <= 0 || cK <= 0) return;
    // triangles of each z-column (in triangle order)
    std::vector<std::vector<int>> column((size_t)cI * cJ);
    for (int t = 0; t < ntri; t++) {
        const V a = m[tris[3 * t]], b = m[tris[3 * t + 1]], e = m[tris[3 * t + 2]];
        const float mn[2] = {std::min(a.x, std::min(b.x, e.x)), std::min(a.y, std::min(b.y, e.y))};
        const double ext[2] = {(double)std::max(a.x, std::max(b.x, e.x)) - mn[0], (double)std::max(a.y, std::max(b.y, e.y)) - mn[1]};
        const int i0 = std::max(floor_index(mn[0], dx), 0), j0 = std::max(floor_index(mn[1], dx), 0);
        const int i1 = std::min(floor_index(mn[0] + (float)ext[0], dx), cI - 1);
        const int j1 = std::min(floor_index(mn[1] + (float)ext[1], dx), cJ - 1);
        for (int j = j0; j <= j1; j++)
            for (int i = i0; i <= i1; i++) column[(size_t)i + (size_t)cI * j].push_back(t);
    }
    const V jitter{(float)(0.00031 * dx), (float)(-0.00047 * dx), (float)(0.00023 * dx)};
    const double hw = 0.5 * dx;
    std::vector<float> zc;
    for (int j = 0; j < cJ; j++)
        for (int i = 0; i < cI; i++) {
            const std::vector<int> &ts = column[(size_t)i + (size_t)cI * j];
            if (ts.empty()) continue;
            const V gp = vadd(V{(float)((float)i * dx + hw), (float)((float)j * dx + hw), (float)((float)-1 * dx + hw)}, jitter);
            zc.clear();
            for (int t : ts) {
                float z;
                if (ray_z_crossing(gp, m[tris[3 * t]], m[tris[3 * t + 1]], m[tris[3 * t + 2]], &z)) zc.push_back(z);
            }
            if (zc.size() % 2 != 0) continue;
            for (int k = 0; k < cK; k++) {
                const float zk = (float)((float)k * dx + hw);
                int less = 0;
                for (float z : zc) less += z < zk;
                if (less % 2 == 1) mark(i + go[0], j + go[1], k + go[2]);
            }
        }
}

// MeshUtils::getGridNodesInsideTriangleMesh(mesh, dx, Array3d<bool>)
// (meshutils.cpp:373-428) over nI x nJ x nK nodes: a mesh inside the grid's
// box [0, (nI-1) dx) x ... is tested whole; otherwise it is cut into its
// connected islands (_splitInsideOutsideMesh, :430-452; _splitIntoMeshIslands,
// :454-557): the islands inside the box together, each island that reaches
// into the box on its own, the rest not at all.
void grid_nodes_inside(const std::vector<V> &vtx, const std::vector<int> &tris, int nI, int nJ, int nK, double dx,
                       std::vector<uint8_t> &inside) {
    inside.assign((size_t)nI * nJ * nK, 0);
    auto mark = [&](int i, int j, int k) {
        if (i >= 0 && j >= 0 && k >= 0 && i < nI && j < nJ && k < nK)
            inside[(size_t)i + (size_t)nI * ((size_t)j + (size_t)nJ * k)] = 1;
    };
    const double W = (double)(nI - 1) * dx, H = (double)(nJ - 1) * dx, D = (double)(nK - 1) * dx;
    auto in_box = [&](V p) {   // AABB::isPointInside (aabb.cpp:130-133), position 0
        return p.x >= 0.0f && p.y >= 0.0f && p.z >= 0.0f && (double)p.x < W && (double)p.y < H && (double)p.z < D;
    };
    bool contained = true;
    for (const V &v : vtx) contained = contained && in_box(v);
    if (contained) {
        inside_nodes_of(vtx, tris, dx, mark);
        return;
    }
    // islands: vertices connected through triangle edges
    const int nv = (int)vtx.size(), ntri = (int)tris.size() / 3;
    std::vector<int> root(nv);
    for (int q = 0; q < nv; q++) root[q] = q;
    auto find = [&](int q) {
        while (root[q] != q) q = root[q] = root[root[q]];
        return q;
    };
    for (int t = 0; t < ntri; t++)
        for (int e = 1; e < 3; e++) {
            const int a = find(tris[3 * t]), b = find(tris[3 * t + e]);
            if (a != b) root[std::max(a, b)] = std::min(a, b);
        }
    std::vector<int> island(nv), count;
    for (int q = 0; q < nv; q++) {
        const int r = find(q);
        if (r == q) { island[q] = (int)count.size(); count.push_back(0); }
        else island[q] = island[r];
        count[island[q]]++;
    }
    const int ni = (int)count.size();
    std::vector<std::vector<V>> iv(ni);
    std::vector<std::vector<int>> it(ni);
    std::vector<int> local(nv);
    for (int q = 0; q < nv; q++) {
        local[q] = (int)iv[island[q]].size();
        iv[island[q]].push_back(vtx[q]);
    }
    for (int t = 0; t < ntri; t++) {
        std::vector<int> &d = it[island[tris[3 * t]]];
        for (int e = 0; e < 3; e++) d.push_back(local[tris[3 * t + e]]);
    }
    std::vector<V> inV;
    std::vector<int> inT;
    for (int g = 0; g < ni; g++) {
        const std::vector<V> &v = iv[g];
        float lo[3] = {v[0].x, v[0].y, v[0].z}, hi[3] = {v[0].x, v[0].y, v[0].z};
        for (const V &p : v) {
            lo[0] = std::min(lo[0], p.x); lo[1] = std::min(lo[1], p.y); lo[2] = std::min(lo[2], p.z);
            hi[0] = std::max(hi[0], p.x); hi[1] = std::max(hi[1], p.y); hi[2] = std::max(hi[2], p.z);
        }
        // AABB of the island: float position, double extent; its max point in float
        const V mn{lo[0], lo[1], lo[2]};
        const V mx{(float)((double)lo[0] + ((double)hi[0] - lo[0])), (float)((double)lo[1] + ((double)hi[1] - lo[1])),
                   (float)((double)lo[2] + ((double)hi[2] - lo[2]))};
        if (in_box(mn) && in_box(mx)) {
            const int base = (int)inV.size();
            inV.insert(inV.end(), v.begin(), v.end());
            for (int idx : it[g]) inT.push_back(base + idx);
        } else {
            // AABB::getIntersection with the grid's box (aabb.cpp:170-190)
            const double bmax[3] = {W, H, D};
            const float vmn[3] = {mn.x, mn.y, mn.z}, vmx[3] = {mx.x, mx.y, mx.z};
            bool apart = false, some = false;
            for (int a = 0; a < 3; a++) {
                const float bx = (float)bmax[a];
                if (vmn[a] > bx || vmx[a] < 0.0f) apart = true;
                const double w = (double)std::min(vmx[a], bx) - (double)std::max(vmn[a], 0.0f);
                some = some || w > 0.0;
            }
            if (!apart && some) inside_nodes_of(v, it[g], dx, mark);
        }
    }
    if (!inV.empty()) inside_nodes_of(inV, inT, dx, mark);
}

// The level set of one mesh over a sub-grid of nI x nJ x nK nodes whose
// first node sits at `origin` (float position): the exact band in the block
// frame and the signs from the nodes inside (meshlevelset.cpp:572-601,
// 781-1158, 1298-1316).  Vertices are already relative to `origin`.
void mesh_level_set(const std::vector<V> &vtx, const std::vector<int> &tris, int nI, int nJ, int nK, double dx,
                    int band, std::vector<float> &phi, std::vector<int> &tri) {
    const float upper = (float)((double)(nI + nJ + nK) * dx);
    auto nid = [&](int i, int j, int k) { return (size_t)i + (size_t)nI * ((size_t)j + (size_t)nJ * k); };
    phi.assign((size_t)nI * nJ * nK, upper);
    tri.assign(phi.size(), -1);
    const int bw = 10;
    const int ntri = (int)tris.size() / 3;
    for (int t = 0; t < ntri; t++) {
        const V a = vtx[tris[3 * t]], b = vtx[tris[3 * t + 1]], e = vtx[tris[3 * t + 2]];
        // AABB of the triangle: float minimum, double extent (aabb.cpp:84-110)
        const float mn[3] = {std::min(a.x, std::min(b.x, e.x)), std::min(a.y, std::min(b.y, e.y)), std::min(a.z, std::min(b.z, e.z))};
        const double ext[3] = {(double)std::max(a.x, std::max(b.x, e.x)) - mn[0], (double)std::max(a.y, std::max(b.y, e.y)) - mn[1],
                               (double)std::max(a.z, std::max(b.z, e.z)) - mn[2]};
        int lo[3], hi[3];
        const int n[3] = {nI, nJ, nK};
        bool outside = false;
        for (int q = 0; q < 3; q++) {
            lo[q] = floor_index(mn[q], dx) - band;
            hi[q] = floor_index(mn[q] + (float)ext[q], dx) + band + 1;
            if (hi[q] < 0 || lo[q] >= n[q]) outside = true;
            lo[q] = std::max(lo[q], 0);
            hi[q] = std::min(hi[q], n[q] - 1);
        }
        if (outside) continue;
        for (int k = lo[2]; k <= hi[2]; k++)
            for (int j = lo[1]; j <= hi[1]; j++)
                for (int i = lo[0]; i <= hi[0]; i++) {
                    const V off{gpos(i / bw, (double)bw * dx), gpos(j / bw, (double)bw * dx), gpos(k / bw, (double)bw * dx)};
                    const V g{gpos(i % bw, dx), gpos(j % bw, dx), gpos(k % bw, dx)};
                    const float dist = vlen(vsub(closest_point(g, vsub(a, off), vsub(b, off), vsub(e, off)), g));
                    const size_t id = nid(i, j, k);
                    if (dist < phi[id]) {
                        phi[id] = dist;
                        tri[id] = t;
                    }
                }
    }
    std::vector<uint8_t> inside;
    grid_nodes_inside(vtx, tris, nI, nJ, nK, dx, inside);
    for (size_t q = 0; q < phi.size(); q++)
        if (inside[q]) phi[q] = -phi[q];
}

}  // namespace

void DomainBox::compute(int I_, int J_, int K_, double dx_, double cfl, const std::vector<MeshObstacle> &obstacles) {
    I = I_; J = J_; K = K_; dx = dx_;
    // boundary box: AABB::expand(-3dx - 1e-4): position -= h, extent += v
    double v = -3 * dx - 1e-4, h = 0.5 * v;
    px = 0.0f - (float)h; py = 0.0f - (float)h; pz = 0.0f - (float)h;
    ex = I * dx + v; ey = J * dx + v; ez = K * dx + v;
    const int ni = I + 1, nj = J + 1, nk = K + 1;
    const float upper = (float)((double)(ni + nj + nk) * dx);
    nodal.assign((size_t)ni * nj * nk, upper);
    nodeObject.assign(nodal.size(), -1);
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
                    if (dist < cur) {
                        cur = dist;
                        nodeObject[nidx(i, j, k)] = 0;   // the domain walls
                    }
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

    // static mesh obstacles: each one's level set over its sub-grid, unioned
    // into a temporary full-grid level set, which is unioned into the walls'
    // (a node takes the smaller value; its closest object changes only where
    // the new value is also smaller in magnitude and came from the band)
    for (size_t q = 0; q < obstacles.size(); q++) {
        const MeshObstacle &ob = obstacles[q];
        const int nv = (int)ob.verts.size() / 3;
        if (nv == 0 || ob.tris.empty()) continue;
        std::vector<V> wv(nv);
        for (int v = 0; v < nv; v++) wv[v] = V{ob.verts[3 * v], ob.verts[3 * v + 1], ob.verts[3 * v + 2]};
        float lo[3] = {wv[0].x, wv[0].y, wv[0].z}, hi[3] = {wv[0].x, wv[0].y, wv[0].z};
        for (const V &v : wv) {
            lo[0] = std::min(lo[0], v.x); lo[1] = std::min(lo[1], v.y); lo[2] = std::min(lo[2], v.z);
            hi[0] = std::max(hi[0], v.x); hi[1] = std::max(hi[1], v.y); hi[2] = std::max(hi[2], v.z);
        }
        const double ext[3] = {(double)hi[0] - lo[0], (double)hi[1] - lo[1], (double)hi[2] - lo[2]};
        const int cells[3] = {I, J, K};
        int g0[3], g1[3];
        for (int a = 0; a < 3; a++) {   // meshobject.cpp:528-536
            g0[a] = std::max(floor_index(lo[a], dx) - band, 0);
            g1[a] = std::min(floor_index(lo[a] + (float)ext[a], dx) + band + 1, cells[a] - 1);
        }
        const int gw = g1[0] - g0[0], gh = g1[1] - g0[1], gd = g1[2] - g0[2];
        if (gw <= 0 || gh <= 0 || gd <= 0) continue;   // outside the domain
        const V origin{gpos(g0[0], dx), gpos(g0[1], dx), gpos(g0[2], dx)};
        std::vector<V> rel(nv);
        for (int v = 0; v < nv; v++) rel[v] = vsub(wv[v], origin);
        std::vector<float> iphi;
        std::vector<int> itri;
        mesh_level_set(rel, ob.tris, gw + 1, gh + 1, gd + 1, dx, band, iphi, itri);
        // island -> temporary level set -> solid level set
        std::vector<float> tphi(nodal.size(), upper);
        std::vector<int> tobj(nodal.size(), -1);
        for (int k = 0; k <= gd; k++)
            for (int j = 0; j <= gh; j++)
                for (int i = 0; i <= gw; i++) {
                    const int a = i + g0[0], b = j + g0[1], c = k + g0[2];
                    if (a > I || b > J || c > K) continue;
                    const size_t s = (size_t)i + (size_t)(gw + 1) * ((size_t)j + (size_t)(gh + 1) * k);
                    const size_t d = nidx(a, b, c);
                    if (iphi[s] < tphi[d]) {
                        if (std::fabs(iphi[s]) < std::fabs(tphi[d]) && itri[s] != -1) tobj[d] = (int)q + 1;
                        tphi[d] = iphi[s];
                    }
                }
        for (size_t d = 0; d < nodal.size(); d++) {
            if (tphi[d] < nodal[d]) {
                if (std::fabs(tphi[d]) < std::fabs(nodal[d]) && tobj[d] != -1) nodeObject[d] = tobj[d];
                nodal[d] = tphi[d];
            }
        }
    }
    nodeFriction.assign(nodal.size(), 0.0f);
    anyFriction = false;
    for (size_t d = 0; d < nodal.size(); d++) {
        const int o = nodeObject[d];
        nodeFriction[d] = o > 0 ? obstacles[o - 1].friction : 0.0f;   // the walls have no friction
        anyFriction = anyFriction || nodeFriction[d] != 0.0f;
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

    // face friction: the mean of its four nodes' (fluidsimulation.cpp:3785-3846)
    auto F = [&](int i, int j, int k) { return nodeFriction[nidx(i, j, k)]; };
    auto mean4 = [](float a, float b, float c, float d) {
        float f = 0.0f;
        f += a;
        f += b;
        f += c;
        f += d;
        return 0.25f * f;
    };
    fu.assign(wu.size(), 0.0f);
    fv.assign(wv.size(), 0.0f);
    fw.assign(ww.size(), 0.0f);
    if (anyFriction) {
        for (int k = 0; k < K; k++)
            for (int j = 0; j < J; j++)
                for (int i = 0; i <= I; i++)
                    fu[(size_t)i + (size_t)(I + 1) * ((size_t)j + (size_t)J * k)] =
                        mean4(F(i, j, k), F(i, j + 1, k), F(i, j, k + 1), F(i, j + 1, k + 1));
        for (int k = 0; k < K; k++)
            for (int j = 0; j <= J; j++)
                for (int i = 0; i < I; i++)
                    fv[(size_t)i + (size_t)I * ((size_t)j + (size_t)(J + 1) * k)] =
                        mean4(F(i, j, k), F(i + 1, j, k), F(i, j, k + 1), F(i + 1, j, k + 1));
        for (int k = 0; k <= K; k++)
            for (int j = 0; j < J; j++)
                for (int i = 0; i < I; i++)
                    fw[(size_t)i + (size_t)I * ((size_t)j + (size_t)J * k)] =
                        mean4(F(i, j, k), F(i + 1, j, k), F(i, j + 1, k), F(i + 1, j + 1, k));
    }

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

// The inputs of seeding a fluid mesh (_updateAddedFluidMeshObjectQueue,
// fluidsimulation.cpp:4724-4759): the cells around the grid nodes inside the
// mesh (MeshObject::getCells, meshobject.cpp:101-140; the eight cells that
// share a node, grid3d.h getVertexGridIndexNeighbours) and the mesh's level
// set over the whole grid's nodes, exact in a band of 3
// (MeshLevelSet::fastCalculateSignedDistanceField, meshlevelset.cpp:572-601;
// outside the band the upper bound, negated inside).
void mesh_fluid_cells(int I, int J, int K, double dx, const std::vector<float> &verts, const std::vector<int> &tris,
                      std::vector<int> &cells, std::vector<float> &phi) {
    const int nv = (int)verts.size() / 3;
    std::vector<V> wv(nv);
    for (int v = 0; v < nv; v++) wv[v] = V{verts[3 * v], verts[3 * v + 1], verts[3 * v + 2]};
    std::vector<uint8_t> nodes;
    grid_nodes_inside(wv, tris, I + 1, J + 1, K + 1, dx, nodes);
    std::vector<uint8_t> mark((size_t)I * J * K, 0);
    for (int k = 0; k <= K; k++)
        for (int j = 0; j <= J; j++)
            for (int i = 0; i <= I; i++) {
                if (!nodes[(size_t)i + (size_t)(I + 1) * ((size_t)j + (size_t)(J + 1) * k)]) continue;
                for (int c = k - 1; c <= k; c++)
                    for (int b = j - 1; b <= j; b++)
                        for (int a = i - 1; a <= i; a++)
                            if (a >= 0 && b >= 0 && c >= 0 && a < I && b < J && c < K)
                                mark[(size_t)a + (size_t)I * ((size_t)b + (size_t)J * c)] = 1;
            }
    cells.clear();
    for (size_t q = 0; q < mark.size(); q++)
        if (mark[q]) cells.push_back((int)q);
    std::vector<int> tri;
    mesh_level_set(wv, tris, I + 1, J + 1, K + 1, dx, 3, phi, tri);
}

// MeshFluidSource::update for a static mesh (meshfluidsource.cpp:171-214)
// with _getGridBoundsFromTriangleMesh (:300-318): the mesh's AABB (double
// extent plus 1e-9, aabb.cpp:54-82), expanded by 4 dx, its corners' cells
// clamped to the grid give the sub-grid; a mesh whose box meets the domain
// box (I+1, J+1, K+1 cells) in less than dx^3 / 8 leaves an empty level set.
void fluid_source_setup(int I, int J, int K, double dx, const std::vector<float> &verts, const std::vector<int> &tris,
                        SourceGrid &g) {
    const int nv = (int)verts.size() / 3;
    std::vector<V> wv(nv);
    for (int v = 0; v < nv; v++) wv[v] = V{verts[3 * v], verts[3 * v + 1], verts[3 * v + 2]};
    // MeshObject::getCells (meshobject.cpp:101-140)
    std::vector<uint8_t> nodes;
    grid_nodes_inside(wv, tris, I + 1, J + 1, K + 1, dx, nodes);
    std::vector<uint8_t> mark((size_t)I * J * K, 0);
    for (int k = 0; k <= K; k++)
        for (int j = 0; j <= J; j++)
            for (int i = 0; i <= I; i++) {
                if (!nodes[(size_t)i + (size_t)(I + 1) * ((size_t)j + (size_t)(J + 1) * k)]) continue;
                for (int c = k - 1; c <= k; c++)
                    for (int b = j - 1; b <= j; b++)
                        for (int a = i - 1; a <= i; a++)
                            if (a >= 0 && b >= 0 && c >= 0 && a < I && b < J && c < K)
                                mark[(size_t)a + (size_t)I * ((size_t)b + (size_t)J * c)] = 1;
            }
    g.cells.clear();
    for (size_t q = 0; q < mark.size(); q++)
        if (mark[q]) g.cells.push_back((int)q);
    // the mesh's AABB
    double mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
    for (int v = 0; v < nv; v++) {
        const double p[3] = {wv[v].x, wv[v].y, wv[v].z};
        for (int a = 0; a < 3; a++) {
            mn[a] = v == 0 ? p[a] : std::fmin(p[a], mn[a]);
            mx[a] = v == 0 ? p[a] : std::fmax(p[a], mx[a]);
        }
    }
    float pos[3];
    double ext[3];
    for (int a = 0; a < 3; a++) {
        pos[a] = (float)mn[a];
        ext[a] = nv > 0 ? mx[a] - mn[a] + 1e-9 : 0.0;
    }
    // expand(4 dx), corners, cells
    const double pad = 4.0 * dx, h = 0.5 * pad;
    const int n[3] = {I, J, K};
    int gmax[3];
    for (int a = 0; a < 3; a++) {
        const float lo = pos[a] - (float)h;
        const float hi = lo + (float)(ext[a] + pad);
        const int g0 = floor_index(lo, dx), g1 = floor_index(hi, dx);
        g.gmin[a] = (int)std::fmax(g0, 0);
        gmax[a] = (int)std::fmin(g1, n[a] - 1);
        g.offset[a] = gpos(g.gmin[a], dx);
        g.nodes[a] = std::max(gmax[a] - g.gmin[a] + 1, 1) + 1;
    }
    // AABB::isIntersecting(domain box, dx^3 / 8) (aabb.cpp:170-195)
    bool meets = true;
    double vol = 1.0;
    for (int a = 0; a < 3; a++) {
        const float lo1 = pos[a], hi1 = pos[a] + (float)ext[a];
        const float lo2 = 0.0f, hi2 = (float)((n[a] + 1) * dx);
        if (lo1 > hi2 || hi1 < lo2) meets = false;
        vol *= (double)std::fmin(hi1, hi2) - (double)std::fmax(lo1, lo2);
    }
    meets = meets && vol > (dx * dx * dx) * 0.125;
    std::vector<V> local;
    std::vector<int> ltris;
    if (meets) {
        local.resize(nv);
        for (int v = 0; v < nv; v++)
            local[v] = V{wv[v].x + (-g.offset[0]), wv[v].y + (-g.offset[1]), wv[v].z + (-g.offset[2])};
        ltris = tris;
    }
    std::vector<int> tri;
    mesh_level_set(local, ltris, g.nodes[0], g.nodes[1], g.nodes[2], dx, 2, g.phi, tri);
}

}  // namespace flip
