// Surface reconstruction for getIsomesh(): the marker particles' implicit
// surface, polygonised by marching cubes on a grid subdivided `s` times,
// then smoothed.  This restates, on the GPU, what the reference's mesher
// thread does at the first substep of every frame
// (FluidSimulation::_outputSurfaceMeshThread, fluidsimulation.cpp:5150-5219):
//
//   ParticleMesher::meshParticles (particlemesher.cpp:35-55) with one compute
//   chunk: the 10-node blocks that hold particles, feathered by one block
//   (:116-137); the chunk around them (:139-282); per node the smallest
//   |node - p| - r over the particles whose search box covers it, in the
//   frame of the node's block (:406-549, :618-664), negated (:472-478);
//   ScalarField's clamp of solid nodes to the surface threshold
//   (scalarfield.cpp:372-448); Polygonizer3d (polygonizer3d.cpp:380-675):
//   cells with nodes on both sides, vertices on cut edges placed by linear
//   interpolation and kept out of the solid (:455-491), numbered in the order
//   the reference's scan over cells and edges creates them; triangles from
//   the marching-cubes table; the chunk offset and the scale/unscale of
//   meshParticles; TriangleMesh::smooth (trianglemesh.cpp:481-585).
//
// The GPU work is organised for parallelism, not as the reference's loops:
//   * field: one CTA per 10^3-node block, particles found through the cell
//     bins, each particle's node box scattered into the block's shared
//     memory with an atomic minimum of squared distances (sqrt and the
//     subtraction of r are monotone, so min(|d|) - r comes out exactly);
//   * numbering: a vertex belongs to the first cell in flat order that holds
//     its edge (for an edge, the cell below it in every perpendicular axis
//     where there is one).  So a cell's new vertices and its triangles are
//     counted from its cube index and position alone; a scan over cells
//     gives every cell its first vertex and triangle, and the vertex of any
//     edge is found from the cell that creates it.  The numbering is the
//     reference's, with no sequential pass;
//   * smoothing: vertex -> triangle lists by counting sort, each list sorted
//     by triangle index so the neighbour sums add in the reference's order.
// Arithmetic follows the reference operation by operation (the library is
// built with --fmad=false): float distances, FP64 interpolation fractions
// and solid-level-set samples, float vertex arithmetic.  Vertices and
// triangles come out identical to the reference's for the same particles.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/flip3d.h"
#include "flip_device.cuh"

namespace flip {
namespace {

constexpr int MB = 10;          // ParticleMesher::_blockwidth (particlemesher.h:190)
constexpr int MESH_TPB = 256;
constexpr int CELLS_PER_THREAD = 8;
constexpr int TILE = MESH_TPB * CELLS_PER_THREAD;   // cells per scan tile

// The marching-cubes triangle table (Lorensen and Cline's cases as Paul
// Bourke published them, the table the reference's Polygonizer3d uses,
// polygonizer3d.cpp:97-354), re-encoded: case q's triangles are the edge ids
// in the 4-bit fields of kTri[q], lowest first, three per triangle, ended by
// 0xF.  The edge table is not stored: edge e is cut when its two corners
// differ in the cube index.
__constant__ unsigned long long kTri[256] = {
    0xffffffffffffffffull, 0xfffffffffffff380ull, 0xfffffffffffff910ull, 0xffffffffff189381ull,
    0xfffffffffffffa21ull, 0xffffffffffa21380ull, 0xffffffffff920a29ull, 0xfffffff89a8a2382ull,
    0xfffffffffffff2b3ull, 0xffffffffff0b82b0ull, 0xffffffffffb32091ull, 0xfffffffb89b912b1ull,
    0xffffffffff3ab1a3ull, 0xfffffffab8a801a0ull, 0xfffffff9ab9b3093ull, 0xffffffffffb8aa89ull,
    0xfffffffffffff874ull, 0xffffffffff437034ull, 0xffffffffff748910ull, 0xfffffff137174914ull,
    0xffffffffff748a21ull, 0xfffffffa21403743ull, 0xfffffff748209a29ull, 0xffff4973727929a2ull,
    0xffffffffff2b3748ull, 0xfffffff40242b74bull, 0xfffffffb32748109ull, 0xffff1292b9b49b74ull,
    0xfffffff487ab31a3ull, 0xffff4b7401b41ab1ull, 0xffff30bab9b09874ull, 0xfffffffab99b4b74ull,
    0xfffffffffffff459ull, 0xffffffffff380459ull, 0xffffffffff051450ull, 0xfffffff513538458ull,
    0xffffffffff459a21ull, 0xfffffff594a21803ull, 0xfffffff204245a25ull, 0xffff8434535235a2ull,
    0xffffffffffb32459ull, 0xfffffff594b802b0ull, 0xfffffffb32510450ull, 0xffff584b82852512ull,
    0xfffffff45931ab3aull, 0xffffab81a8180594ull, 0xffff30bab5b05045ull, 0xfffffffb8aa85845ull,
    0xffffffffff975879ull, 0xfffffff375359039ull, 0xfffffff751710870ull, 0xffffffffff753351ull,
    0xfffffff21a759879ull, 0xffff37503505921aull, 0xffff25a758528208ull, 0xfffffff7533525a2ull,
    0xfffffff2b3987597ull, 0xffffb72029279759ull, 0xffff751871810b32ull, 0xfffffff51771b12bull,
    0xffffb3a31a758859ull, 0xf0aba010b7905075ull, 0xf07570805a30b0abull, 0xffffffffff5b75abull,
    0xfffffffffffff56aull, 0xffffffffff6a5380ull, 0xffffffffff6a5109ull, 0xfffffff6a5891381ull,
    0xffffffffff162561ull, 0xfffffff803621561ull, 0xfffffff620609569ull, 0xffff823625285895ull,
    0xffffffffff56ab32ull, 0xfffffff56a02b80bull, 0xfffffff6a5b32910ull, 0xffffb892b92916a5ull,
    0xfffffff315356b36ull, 0xffff6b51505b0b80ull, 0xffff9505606306b3ull, 0xfffffff89bb96956ull,
    0xffffffffff8746a5ull, 0xfffffffa56374034ull, 0xfffffff7486a5091ull, 0xffff49737179156aull,
    0xfffffff874156216ull, 0xffff743403625521ull, 0xffff620560509748ull, 0xf962695923497937ull,
    0xfffffff56a4872b3ull, 0xffffb720242746a5ull, 0xffff6a5b32874910ull, 0xf6a54b7b492b9129ull,
    0xffff6b51535b3748ull, 0xfb404b7b016b5b15ull, 0xf74836b630560950ull, 0xffff9b7974b96956ull,
    0xffffffffffa4694aull, 0xfffffff380a946a4ull, 0xfffffff04606a10aull, 0xffffa16468618138ull,
    0xfffffff462421941ull, 0xffff462942921803ull, 0xffffffffff624420ull, 0xfffffff624428238ull,
    0xfffffff32b46a94aull, 0xffff6a4a94b82280ull, 0xffffa164606102b3ull, 0xf1b8b12184a16146ull,
    0xffff36b319639469ull, 0xf14641916b0181b8ull, 0xfffffff4600636b3ull, 0xffffffffff86b846ull,
    0xfffffffa98a876a7ull, 0xffffa76a907a0370ull, 0xffff0818717a176aull, 0xfffffff37117a76aull,
    0xffff768981861621ull, 0xf937390976192962ull, 0xfffffff206607087ull, 0xffffffffff276237ull,
    0xffff76898a86ab32ull, 0xf7a9a76790b72702ull, 0xfb32a767a1871081ull, 0xffff17616a71b12bull,
    0xf63136b619768698ull, 0xffffffffff76b190ull, 0xffff06b0b3607087ull, 0xfffffffffffff6b7ull,
    0xfffffffffffffb67ull, 0xffffffffff67b803ull, 0xffffffffff67b910ull, 0xfffffff67b138918ull,
    0xffffffffff7b621aull, 0xfffffff7b6803a21ull, 0xfffffff7b69a2092ull, 0xffff89a38a3a27b6ull,
    0xffffffffff726327ull, 0xfffffff026067807ull, 0xfffffff910732672ull, 0xffff678891681261ull,
    0xfffffff73171a67aull, 0xffff801781a7167aull, 0xffff7a69a0a70730ull, 0xfffffff9a88a7a67ull,
    0xffffffffff68b486ull, 0xfffffff640603b63ull, 0xfffffff109648b68ull, 0xffff63b139369649ull,
    0xfffffff1a28b6486ull, 0xffff640b60b03a21ull, 0xffff9a2920b648b4ull, 0xf36463b34923a39aull,
    0xfffffff264248328ull, 0xffffffffff264240ull, 0xffff834642432091ull, 0xfffffff642241491ull,
    0xffff1a6648168318ull, 0xfffffff40660a01aull, 0xf39a9303a6834364ull, 0xffffffffff4a649aull,
    0xffffffffffb67594ull, 0xfffffff67b594380ull, 0xfffffffb67045105ull, 0xffff51345343867bull,
    0xfffffffb6721a459ull, 0xffff594380a217b6ull, 0xffff204a24a45b67ull, 0xf67b25a523453843ull,
    0xfffffff945267327ull, 0xffff786260680459ull, 0xffff045051673263ull, 0xf851584812786826ull,
    0xffff73167161a459ull, 0xf459078701671a61ull, 0xfa737a6a305a4a04ull, 0xffffa84a458a7a67ull,
    0xfffffff98b9b6596ull, 0xffff590650360b63ull, 0xffffb65510b508b0ull, 0xfffffff1355363b6ull,
    0xffff65b8b9b59a21ull, 0xfa21965690b603b0ull, 0xf52025a50865b58bull, 0xffff35a3a25363b6ull,
    0xffff283265825985ull, 0xfffffff260069659ull, 0xf826283865081851ull, 0xffffffffff612651ull,
    0xf698965683a61631ull, 0xffff06505960a01aull, 0xffffffffffa65830ull, 0xfffffffffffff65aull,
    0xffffffffffb57a5bull, 0xfffffff03857ba5bull, 0xfffffff091ba57b5ull, 0xffff1381897ba57aull,
    0xfffffff15717b21bull, 0xffffb27571721380ull, 0xffff7b2209729579ull, 0xf289823295b27257ull,
    0xfffffff573532a52ull, 0xffff52a578258028ull, 0xffff2a37353a5109ull, 0xf25752a278129289ull,
    0xffffffffff573531ull, 0xfffffff571170780ull, 0xfffffff735539309ull, 0xffffffffff795789ull,
    0xfffffff8ba8a5485ull, 0xffff03bba50b5405ull, 0xffff54aba8a48910ull, 0xf41314943b54a4baull,
    0xffff8548b2582152ull, 0xfb151b2b543b0b40ull, 0xf58b8545b2950520ull, 0xffffffffff3b2549ull,
    0xffff483543253a52ull, 0xfffffff0244252a5ull, 0xf910854583a532a3ull, 0xffff2492914252a5ull,
    0xfffffff153358548ull, 0xffffffffff501540ull, 0xffff530509358548ull, 0xfffffffffffff549ull,
    0xfffffffba9b947b4ull, 0xffffba97b9794380ull, 0xffffb470414b1ba1ull, 0xf4bab474a1843413ull,
    0xffff219b294b97b4ull, 0xf3801b2b197b9479ull, 0xfffffff04224b47bull, 0xffff42343824b47bull,
    0xffff947732972a92ull, 0xf70207872a4797a9ull, 0xfa040a1a472a3a73ull, 0xffffffffff4782a1ull,
    0xfffffff317714194ull, 0xffff178180714194ull, 0xffffffffff347304ull, 0xfffffffffffff784ull,
    0xffffffffff8ba8a9ull, 0xfffffffa9bb93903ull, 0xfffffffba88a0a10ull, 0xffffffffffa3ba13ull,
    0xfffffff8b99b1b21ull, 0xffff9b2921b93903ull, 0xffffffffffb08b20ull, 0xfffffffffffffb23ull,
    0xfffffff98aa82832ull, 0xffffffffff2902a9ull, 0xffff8a1810a82832ull, 0xfffffffffffff2a1ull,
    0xffffffffff819831ull, 0xfffffffffffff190ull, 0xfffffffffffff830ull, 0xffffffffffffffffull,
};

// Cube corners (Grid3d::getGridIndexVertices, grid3d.h:304-313): corner q at
// (i + kCx[q], j + kCy[q], k + kCz[q]).
__constant__ int kCx[8] = {0, 1, 1, 0, 0, 1, 1, 0};
__constant__ int kCy[8] = {0, 0, 0, 0, 1, 1, 1, 1};
__constant__ int kCz[8] = {0, 0, 1, 1, 0, 0, 1, 1};
// Edges in the reference's order (polygonizer3d.cpp:495-630): the corners
// interpolated from and to, the axis of the edge and the corner it starts
// from along that axis (which names the edge in the grid of edges).
__constant__ int kEa[12] = {0, 1, 2, 3, 4, 5, 6, 7, 0, 1, 2, 3};
__constant__ int kEb[12] = {1, 2, 3, 0, 5, 6, 7, 4, 4, 5, 6, 7};
__constant__ int kEdir[12] = {0, 2, 0, 2, 0, 2, 0, 2, 1, 1, 1, 1};
__constant__ int kEorg[12] = {0, 1, 3, 0, 4, 5, 7, 4, 0, 1, 2, 3};

__device__ __forceinline__ unsigned cut_mask(int q) {
    unsigned m = 0;
#pragma unroll
    for (int e = 0; e < 12; e++)
        if (((q >> kEa[e]) ^ (q >> kEb[e])) & 1) m |= 1u << e;
    return m;
}
__device__ __forceinline__ int tri_count(int q) {
    const unsigned long long w = kTri[q];
    int n = 0;
    while (n < 16 && ((w >> (4 * n)) & 0xF) != 0xF) n++;
    return n / 3;
}
// Edges that cell (i, j, k) creates: the first cell in flat order holding an
// edge is the one below it in each perpendicular axis, where that cell exists.
__device__ __forceinline__ unsigned created_mask(int i, int j, int k) {
    unsigned m = 0;
#pragma unroll
    for (int e = 0; e < 12; e++) {
        const int o = kEorg[e], d = kEdir[e];
        const bool ok = (d == 0 || kCx[o] == 1 || i == 0) && (d == 1 || kCy[o] == 1 || j == 0) &&
                        (d == 2 || kCz[o] == 1 || k == 0);
        if (ok) m |= 1u << e;
    }
    return m;
}

// Nodal solid level set at a point, in FP64 as Interpolation::
// trilinearInterpolate(vec3, dx, grid) evaluates it (interpolation.cpp:61-113):
// the cell by floor(p / dx), the offset from the cell's float corner, the
// eight weights; nodes outside the grid count as 0.
__device__ double solid_sample(const MeshFrame &m, const float *S, float px, float py, float pz) {
    const int i = (int)floor((double)px * m.invdx), j = (int)floor((double)py * m.invdx),
              k = (int)floor((double)pz * m.invdx);
    const float gx = (float)((double)(float)i * m.dx), gy = (float)((double)(float)j * m.dx),
                gz = (float)((double)(float)k * m.dx);
    const double x = (double)__fsub_rn(px, gx) * m.invdx, y = (double)__fsub_rn(py, gy) * m.invdx,
                 z = (double)__fsub_rn(pz, gz) * m.invdx;
    const int ni = m.I + 1, nj = m.J + 1, nk = m.K + 1;
    auto at = [&](int a, int b, int c) -> double {
        return (a >= 0 && b >= 0 && c >= 0 && a < ni && b < nj && c < nk)
                   ? (double)S[(long long)a + (long long)ni * ((long long)b + (long long)nj * c)]
                   : 0.0;
    };
    const double p0 = at(i, j, k), p1 = at(i + 1, j, k), p2 = at(i, j + 1, k), p3 = at(i, j, k + 1),
                 p4 = at(i + 1, j, k + 1), p5 = at(i, j + 1, k + 1), p6 = at(i + 1, j + 1, k),
                 p7 = at(i + 1, j + 1, k + 1);
    return p0 * (1 - x) * (1 - y) * (1 - z) + p1 * x * (1 - y) * (1 - z) + p2 * (1 - x) * y * (1 - z) +
           p3 * (1 - x) * (1 - y) * z + p4 * x * (1 - y) * z + p5 * (1 - x) * y * z + p6 * x * y * (1 - z) +
           p7 * x * y * z;
}

// Is chunk node (a, b, c) a solid vertex (ScalarField::setSolidSDF,
// scalarfield.cpp:372-395, MeshLevelSet::_trilinearInterpolateSolidGridPointsThread,
// meshlevelset.cpp:309-340)?
__device__ bool solid_vertex(const MeshFrame &m, const float *S, int a, int b, int c) {
    if (m.solidMode == 2)   // the scalar field's grid is the level set's
        return S[(long long)a + (long long)(m.I + 1) * ((long long)b + (long long)(m.J + 1) * c)] < 0.0f;
    if (m.solidMode == 1 && !(a & 1) && !(b & 1) && !(c & 1))   // subdivision 2 at offset 0: even nodes
        return S[(long long)(a >> 1) + (long long)(m.I + 1) * ((long long)(b >> 1) + (long long)(m.J + 1) * (c >> 1))] <
               0.0f;
    const float px = __fadd_rn((float)((double)(float)a * m.subdx), m.offx);
    const float py = __fadd_rn((float)((double)(float)b * m.subdx), m.offy);
    const float pz = __fadd_rn((float)((double)(float)c * m.subdx), m.offz);
    const double d = solid_sample(m, S, px, py, pz);
    return m.solidMode == 1 ? (float)d < 0.0f : d < 0.0;
}

// ---------------------------------------------------------------- occupancy
// Blocks holding a particle (ParticleMesher::
// _initializeComputeChunkDataActiveBlocks, particlemesher.cpp:116-137).
__global__ void k_mesh_occupancy(ParticleSoA p, int n, MeshFrame m, uint8_t *occ) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int bi = exact_floor(p.px[t], m.invBlock, m.invBlockf), bj = exact_floor(p.py[t], m.invBlock, m.invBlockf),
              bk = exact_floor(p.pz[t], m.invBlock, m.invBlockf);
    if (bi >= 0 && bj >= 0 && bk >= 0 && bi < m.nbI && bj < m.nbJ && bk < m.nbK)
        occ[bi + m.nbI * (bj + m.nbJ * bk)] = 1;
}

// -------------------------------------------------------------- scalar field
// One CTA per block of the chunk (chunk-frame block index = blockIdx).
__global__ void __launch_bounds__(MESH_TPB) k_mesh_field(ParticleSoA p, const int *cellStart, MeshFrame m,
                                                         const uint8_t *active, const float *solidPhi,
                                                         float *field) {
    __shared__ unsigned int smin[MB * MB * MB];
    __shared__ float npos[MB];
    __shared__ float4 recs[MESH_TPB / 32][32];   // per warp: a pass's particles {lx, ly, lz, box}
    const int bx = blockIdx.x, by = blockIdx.y, bz = blockIdx.z;
    for (int q = threadIdx.x; q < MB * MB * MB; q += blockDim.x) smin[q] = 0x7f800000u;   // +inf
    if (threadIdx.x < MB) npos[threadIdx.x] = (float)((double)(float)threadIdx.x * m.subdx);
    __syncthreads();
    if (active[bx + m.cbI * (by + m.cbJ * bz)]) {
        // block frame (_scalarFieldProducerThread, particlemesher.cpp:498-549)
        const float bofx = (float)((double)(float)bx * m.blockdx), bofy = (float)((double)(float)by * m.blockdx),
                    bofz = (float)((double)(float)bz * m.blockdx);
        // candidate cells: every particle whose search box can overlap the
        // block (its list holds no other), with slack for rounding
        const double reach = (double)m.sr + 0.01 * m.dx;
        const double lox = (double)m.offx + bx * m.blockdx - reach, hix = (double)m.offx + (bx + 1) * m.blockdx + reach;
        const double loy = (double)m.offy + by * m.blockdx - reach, hiy = (double)m.offy + (by + 1) * m.blockdx + reach;
        const double loz = (double)m.offz + bz * m.blockdx - reach, hiz = (double)m.offz + (bz + 1) * m.blockdx + reach;
        const int x0 = max((int)floor(lox * m.invdx), 0), x1 = min((int)floor(hix * m.invdx), m.I - 1);
        const int y0 = max((int)floor(loy * m.invdx), 0), y1 = min((int)floor(hiy * m.invdx), m.J - 1);
        const int z0 = max((int)floor(loz * m.invdx), 0), z1 = min((int)floor(hiz * m.invdx), m.K - 1);
        const int ny = y1 - y0 + 1, nrows = x1 >= x0 ? ny * (z1 - z0 + 1) : 0;
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
        const float sr = m.sr;
        float4 *wrec = recs[warp];
        // col / n = (col * ceil(2^11 / n)) >> 11, exact for n <= MB and
        // col < n * MB; lane n holds the multiplier
        const int divLane = lane > 0 ? (2048 + lane - 1) / lane : 0;
        for (int row = warp; row < nrows; row += nwarps) {
            const int cy = y0 + row % ny, cz = z0 + row / ny;
            const long long rbase = (long long)m.I * (cy + (long long)m.J * cz);
            const int pb = cellStart[rbase + x0], pe = cellStart[rbase + x1 + 1];
            for (int base = pb; base < pe; base += 32) {
                // phase 1, a lane per particle: is it in this block's list,
                // and which of the block's nodes does its box cover
                const int t = base + lane;
                int ncol = 0, na = 0;
                float4 rec = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                unsigned packed = 0;
                if (t < pe) {
                    const float px = p.px[t], py = p.py[t], pz = p.pz[t];
                    // the chunk's box, expanded (particlemesher.cpp:287-301, aabb.cpp:122-133)
                    const bool in = px >= m.bbx && py >= m.bby && pz >= m.bbz && (double)px < (double)m.bbx + m.bbw &&
                                    (double)py < (double)m.bby + m.bbh && (double)pz < (double)m.bbz + m.bbd;
                    const float cx = __fsub_rn(px, m.offx), cy2 = __fsub_rn(py, m.offy), cz2 = __fsub_rn(pz, m.offz);
                    // the count pass's block lists (particlemesher.cpp:400-446)
                    const int oi = exact_floor(cx, m.invBlockF, m.invBlockFf),
                              oj = exact_floor(cy2, m.invBlockF, m.invBlockFf),
                              ok = exact_floor(cz2, m.invBlockF, m.invBlockFf);
                    const float bpx = (float)((double)(float)oi * (double)m.blockdxF),
                                bpy = (float)((double)(float)oj * (double)m.blockdxF),
                                bpz = (float)((double)(float)ok * (double)m.blockdxF);
                    bool mine;
                    if (__fsub_rn(cx, sr) > bpx && __fsub_rn(cy2, sr) > bpy && __fsub_rn(cz2, sr) > bpz &&
                        __fadd_rn(cx, sr) < __fadd_rn(bpx, m.blockdxF) &&
                        __fadd_rn(cy2, sr) < __fadd_rn(bpy, m.blockdxF) &&
                        __fadd_rn(cz2, sr) < __fadd_rn(bpz, m.blockdxF)) {
                        mine = oi == bx && oj == by && ok == bz;
                    } else {
                        const int i0 = exact_floor(__fsub_rn(cx, sr), m.invBlockF, m.invBlockFf),
                                  i1 = exact_floor(__fadd_rn(cx, sr), m.invBlockF, m.invBlockFf);
                        const int j0 = exact_floor(__fsub_rn(cy2, sr), m.invBlockF, m.invBlockFf),
                                  j1 = exact_floor(__fadd_rn(cy2, sr), m.invBlockF, m.invBlockFf);
                        const int k0 = exact_floor(__fsub_rn(cz2, sr), m.invBlockF, m.invBlockFf),
                                  k1 = exact_floor(__fadd_rn(cz2, sr), m.invBlockF, m.invBlockFf);
                        mine = bx >= i0 && bx <= i1 && by >= j0 && by <= j1 && bz >= k0 && bz <= k1;
                    }
                    if (in && mine) {
                        const float lx = __fsub_rn(cx, bofx), ly = __fsub_rn(cy2, bofy), lz = __fsub_rn(cz2, bofz);
                        const int a0 = max(exact_floor(__fsub_rn(lx, sr), m.invsub, m.invsubf), 0);
                        const int b0 = max(exact_floor(__fsub_rn(ly, sr), m.invsub, m.invsubf), 0);
                        const int c0 = max(exact_floor(__fsub_rn(lz, sr), m.invsub, m.invsubf), 0);
                        const int a1 = min(exact_floor(__fadd_rn(lx, sr), m.invsub, m.invsubf) + 1, MB - 1);
                        const int b1 = min(exact_floor(__fadd_rn(ly, sr), m.invsub, m.invsubf) + 1, MB - 1);
                        const int c1 = min(exact_floor(__fadd_rn(lz, sr), m.invsub, m.invsubf) + 1, MB - 1);
                        if (a1 >= a0 && b1 >= b0 && c1 >= c0) {
                            na = a1 - a0 + 1;
                            ncol = na * (b1 - b0 + 1);
                            packed = (unsigned)a0 | (unsigned)na << 4 | (unsigned)b0 << 8 | (unsigned)c0 << 12 |
                                     (unsigned)c1 << 16;
                            rec = make_float4(lx, ly, lz, 0.0f);
                        }
                    }
                }
                const unsigned div = (unsigned)__shfl_sync(0xffffffffu, divLane, na);
                if (ncol > 0) {
                    rec.w = __uint_as_float(packed | div << 20);
                    wrec[lane] = rec;
                }
                int incl = ncol;   // inclusive prefix sum of the column counts over the lanes
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int v = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += v;
                }
                const int total = __shfl_sync(0xffffffffu, incl, 31);
                __syncwarp();
                // phase 2, a lane per (particle, column of its box along k):
                // the lanes of one step walk distinct columns
                for (int first = 0; first < total; first += 32) {
                    const int item = first + lane;
                    int L = 0;   // the smallest lane whose inclusive sum exceeds item
#pragma unroll
                    for (int step = 16; step > 0; step >>= 1)
                        if (__shfl_sync(0xffffffffu, incl, L + step - 1) <= item) L += step;
                    const int startL = __shfl_sync(0xffffffffu, incl, L) - __shfl_sync(0xffffffffu, ncol, L);
                    if (item < total) {
                        const float4 pr = wrec[L];
                        const unsigned w = __float_as_uint(pr.w);
                        const int a0 = w & 15, nA = (w >> 4) & 15, b0 = (w >> 8) & 15;
                        const int c0 = (w >> 12) & 15, c1 = (w >> 16) & 15;
                        const int col = item - startL;
                        const int bq = (col * (int)(w >> 20)) >> 11;   // col / nA
                        const int aa = a0 + col - bq * nA, bb = b0 + bq;
                        const float ddx = __fsub_rn(npos[aa], pr.x);
                        const float dy = __fsub_rn(npos[bb], pr.y);
                        const float dxy = __fadd_rn(__fmul_rn(ddx, ddx), __fmul_rn(dy, dy));
                        unsigned int *dst = &smin[aa + MB * (bb + MB * c0)];
                        for (int cc = c0; cc <= c1; cc++, dst += MB * MB) {
                            const float dz = __fsub_rn(npos[cc], pr.z);
                            atomicMin(dst, __float_as_uint(__fadd_rn(dxy, __fmul_rn(dz, dz))));
                        }
                    }
                }
                __syncwarp();
            }
        }
    }
    __syncthreads();
    for (int q = threadIdx.x; q < MB * MB * MB; q += blockDim.x) {
        const int a = MB * bx + q % MB, b = MB * by + (q / MB) % MB, c = MB * bz + q / (MB * MB);
        if (a >= m.ni || b >= m.nj || c >= m.nk) continue;
        const unsigned int s = smin[q];
        const float d = s == 0x7f800000u ? m.maxd : fminf(m.maxd, __fsub_rn(__fsqrt_rn(__uint_as_float(s)), m.r));
        float f = -d;
        if (f > 0.0f && solid_vertex(m, solidPhi, a, b, c)) f = 0.0f;
        field[(long long)a + (long long)m.ni * ((long long)b + (long long)m.nj * c)] = f;
    }
}

// ------------------------------------------------------------------- cells
__device__ __forceinline__ float fld(const MeshFrame &m, const float *F, int a, int b, int c) {
    return F[(long long)a + (long long)m.ni * ((long long)b + (long long)m.nj * c)];
}
__device__ __forceinline__ int cube_index(const MeshFrame &m, const float *F, int i, int j, int k) {
    int q = 0;
#pragma unroll
    for (int v = 0; v < 8; v++)
        if (fld(m, F, i + kCx[v], j + kCy[v], k + kCz[v]) > 0.0f) q |= 1 << v;
    return q;
}

// inclusive warp scan of int2, then the block's exclusive prefix and total
__device__ int2 block_scan_int2(int2 v, int2 *total) {
    __shared__ int2 wsum[MESH_TPB / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int2 x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int a = __shfl_up_sync(0xffffffffu, x.x, o), b = __shfl_up_sync(0xffffffffu, x.y, o);
        if (lane >= o) { x.x += a; x.y += b; }
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    int2 before = make_int2(0, 0), tot = make_int2(0, 0);
    for (int w = 0; w < MESH_TPB / 32; w++) {
        if (w < warp) { before.x += wsum[w].x; before.y += wsum[w].y; }
        tot.x += wsum[w].x;
        tot.y += wsum[w].y;
    }
    __syncthreads();
    *total = tot;
    return make_int2(before.x + x.x - v.x, before.y + x.y - v.y);
}

// Per cell: cube index; per tile: vertices created and triangles.
__global__ void __launch_bounds__(MESH_TPB) k_mesh_count(MeshFrame m, const float *F, long long ncells,
                                                         uint8_t *cube, int2 *tileSums) {
    const long long base = (long long)blockIdx.x * TILE + (long long)threadIdx.x * CELLS_PER_THREAD;
    int2 own = make_int2(0, 0);
    const int ci = m.ni - 1, cj = m.nj - 1;
    for (int q = 0; q < CELLS_PER_THREAD; q++) {
        const long long c = base + q;
        if (c >= ncells) break;
        int i, j, k;
        unflatten(c, ci, cj, i, j, k);
        const int cq = cube_index(m, F, i, j, k);
        cube[c] = (uint8_t)cq;
        if (cq != 0 && cq != 255) {
            own.x += __popc(cut_mask(cq) & created_mask(i, j, k));
            own.y += tri_count(cq);
        }
    }
    int2 tot;
    block_scan_int2(own, &tot);
    if (threadIdx.x == 0) tileSums[blockIdx.x] = tot;
}

// Exclusive scan of the tile sums in place (one CTA, any number of tiles);
// the totals to totals[0..1].
__global__ void k_mesh_scan_tiles(int2 *tileSums, int ntiles, int *totals) {
    __shared__ int2 carry;
    if (threadIdx.x == 0) carry = make_int2(0, 0);
    __syncthreads();
    for (int b0 = 0; b0 < ntiles; b0 += MESH_TPB) {
        const int t = b0 + threadIdx.x;
        const int2 v = t < ntiles ? tileSums[t] : make_int2(0, 0);
        int2 tot;
        const int2 ex = block_scan_int2(v, &tot);
        const int2 cr = carry;
        if (t < ntiles) tileSums[t] = make_int2(cr.x + ex.x, cr.y + ex.y);
        __syncthreads();
        if (threadIdx.x == 0) carry = make_int2(cr.x + tot.x, cr.y + tot.y);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        totals[0] = carry.x;
        totals[1] = carry.y;
    }
}

// Polygonizer3d::_vertexInterp (polygonizer3d.cpp:455-491): the point where
// the field crosses the threshold on the edge from corner 1 to corner 2,
// kept on the liquid side of a solid crossing.
__device__ void vertex_interp(const MeshFrame &m, const float *S, float p1x, float p1y, float p1z, float p2x,
                              float p2y, float p2z, double v1, double v2, float *out) {
    double minmu = 0.0, maxmu = 1.0;
    const double eps = 1e-10;
    const double s1 = (double)(float)solid_sample(m, S, __fadd_rn(p1x, m.offx), __fadd_rn(p1y, m.offy),
                                                  __fadd_rn(p1z, m.offz));
    const double s2 = (double)(float)solid_sample(m, S, __fadd_rn(p2x, m.offx), __fadd_rn(p2y, m.offy),
                                                  __fadd_rn(p2z, m.offz));
    if ((s1 < 0.0 && s2 >= 0.0) || (s2 < 0.0 && s1 >= 0.0)) {
        const double diff = s2 - s1;
        if (fabs(diff) > eps) {
            const double su = -s1 / diff;
            if (s1 < 0.0) minmu = su;
            else maxmu = su;
        } else {
            maxmu = minmu;
        }
    }
    minmu = fmax(minmu, eps);
    maxmu = fmin(maxmu, 1.0 - eps);
    double mu = (0.0 - v1) / (v2 - v1);
    if (mu < minmu) mu = minmu;
    if (mu > maxmu) mu = maxmu;
    const float fm = (float)mu;
    out[0] = __fadd_rn(p1x, __fmul_rn(fm, __fsub_rn(p2x, p1x)));
    out[1] = __fadd_rn(p1y, __fmul_rn(fm, __fsub_rn(p2y, p1y)));
    out[2] = __fadd_rn(p1z, __fmul_rn(fm, __fsub_rn(p2z, p1z)));
}

// Every cell's first vertex and triangle; the vertices it creates, moved to
// the simulation's frame (translate by the chunk offset, scale, unscale:
// particlemesher.cpp:35-55, 271-280).
__global__ void __launch_bounds__(MESH_TPB) k_mesh_vertices(MeshFrame m, const float *F, const float *S,
                                                            long long ncells, const uint8_t *cube,
                                                            const int2 *tileBase, int *vstart, int *tstart,
                                                            float *verts) {
    const long long base = (long long)blockIdx.x * TILE + (long long)threadIdx.x * CELLS_PER_THREAD;
    const int ci = m.ni - 1, cj = m.nj - 1;
    int2 own = make_int2(0, 0);
    for (int q = 0; q < CELLS_PER_THREAD; q++) {
        const long long c = base + q;
        if (c >= ncells) break;
        const int cq = cube[c];
        if (cq != 0 && cq != 255) {
            int i, j, k;
            unflatten(c, ci, cj, i, j, k);
            own.x += __popc(cut_mask(cq) & created_mask(i, j, k));
            own.y += tri_count(cq);
        }
    }
    int2 tot;
    int2 run = block_scan_int2(own, &tot);
    const int2 tb = tileBase[blockIdx.x];
    run.x += tb.x;
    run.y += tb.y;
    const float sdx = (float)m.subdx;
    for (int q = 0; q < CELLS_PER_THREAD; q++) {
        const long long c = base + q;
        if (c >= ncells) break;
        vstart[c] = run.x;
        tstart[c] = run.y;
        const int cq = cube[c];
        if (cq == 0 || cq == 255) continue;
        int i, j, k;
        unflatten(c, ci, cj, i, j, k);
        const unsigned mk = cut_mask(cq) & created_mask(i, j, k);
        for (int e = 0; e < 12; e++) {
            if (!(mk >> e & 1u)) continue;
            const int A = kEa[e], B = kEb[e];
            const int ai = i + kCx[A], aj = j + kCy[A], ak = k + kCz[A];
            const int bi = i + kCx[B], bj = j + kCy[B], bk = k + kCz[B];
            float v[3];
            // Polygonizer3d::_getVertexPosition (polygonizer3d.cpp:356-359)
            vertex_interp(m, S, __fmul_rn(sdx, (float)ai), __fmul_rn(sdx, (float)aj), __fmul_rn(sdx, (float)ak),
                          __fmul_rn(sdx, (float)bi), __fmul_rn(sdx, (float)bj), __fmul_rn(sdx, (float)bk),
                          (double)fld(m, F, ai, aj, ak), (double)fld(m, F, bi, bj, bk), v);
            float *o = verts + 3LL * run.x;
            o[0] = __fmul_rn(__fmul_rn(__fadd_rn(v[0], m.offx), m.scalef), m.invscalef);
            o[1] = __fmul_rn(__fmul_rn(__fadd_rn(v[1], m.offy), m.scalef), m.invscalef);
            o[2] = __fmul_rn(__fmul_rn(__fadd_rn(v[2], m.offz), m.scalef), m.invscalef);
            run.x++;
        }
        run.y += tri_count(cq);
    }
}

// The vertex on edge e of cell (i, j, k): the cell that creates it, the
// edge's number there, and its rank among that cell's new vertices.
__device__ int edge_vertex(const MeshFrame &m, const uint8_t *cube, const int *vstart, int i, int j, int k, int e) {
    const int o = kEorg[e], d = kEdir[e];
    const int ni = i + kCx[o], nj = j + kCy[o], nk = k + kCz[o];   // the edge's first node
    const int pi = d == 0 ? ni : max(ni - 1, 0), pj = d == 1 ? nj : max(nj - 1, 0), pk = d == 2 ? nk : max(nk - 1, 0);
    const int ox = ni - pi, oy = nj - pj, oz = nk - pk;   // the node's corner offset in the creating cell
    int e2 = 0;
#pragma unroll
    for (int f = 0; f < 12; f++) {
        const int of = kEorg[f];
        if (kEdir[f] == d && kCx[of] == ox && kCy[of] == oy && kCz[of] == oz) e2 = f;
    }
    const long long c2 = (long long)pi + (long long)(m.ni - 1) * ((long long)pj + (long long)(m.nj - 1) * pk);
    const unsigned mk = cut_mask(cube[c2]) & created_mask(pi, pj, pk);
    return vstart[c2] + __popc(mk & ((1u << e2) - 1u));
}

// Polygonizer3d::_polygonizeCell (polygonizer3d.cpp:635-656)
__global__ void k_mesh_triangles(MeshFrame m, long long ncells, const uint8_t *cube, const int *vstart,
                                 const int *tstart, int *tris) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    const int cq = cube[c];
    if (cq == 0 || cq == 255) return;
    int i, j, k;
    unflatten(c, m.ni - 1, m.nj - 1, i, j, k);
    const unsigned long long w = kTri[cq];
    int *o = tris + 3LL * tstart[c];
    for (int t = 0; t < 15; t++) {
        const int e = (int)((w >> (4 * t)) & 0xF);
        if (e == 0xF) break;
        o[t] = edge_vertex(m, cube, vstart, i, j, k, e);
    }
}

// -------------------------------------------------------------- smoothing
// TriangleMesh::_updateVertexTriangles (trianglemesh.cpp:481-499): each
// vertex's triangles in ascending order.
__global__ void k_mesh_adj_count(const int *tris, int ntris, int2 *count) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * ntris) return;
    atomicAdd(&count[tris[t]].x, 1);
}
__global__ void k_mesh_adj_fill(const int *tris, int ntris, const int2 *start, int *cursor, int *list) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * ntris) return;
    const int v = tris[t];
    list[start[v].x + atomicAdd(&cursor[v], 1)] = t / 3;
}
__global__ void k_mesh_adj_sort(const int2 *start, int nverts, int *list) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nverts) return;
    const int b = start[v].x, e = start[v + 1].x;
    for (int a = b + 1; a < e; a++) {
        const int key = list[a];
        int q = a - 1;
        while (q >= b && list[q] > key) {
            list[q + 1] = list[q];
            q--;
        }
        list[q + 1] = key;
    }
}
// TriangleMesh::_smoothTriangleMesh (trianglemesh.cpp:536-570): the mean of
// the other corners of the vertex's triangles, then v + value (mean - v).
__global__ void k_mesh_smooth(const float *vin, float *vout, const int *tris, const int2 *start, const int *list,
                              int nverts, float value) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nverts) return;
    float ax = 0.0f, ay = 0.0f, az = 0.0f;
    int count = 0;
    for (int q = start[v].x; q < start[v + 1].x; q++) {
        const int *t = tris + 3LL * list[q];
        for (int s = 0; s < 3; s++) {
            const int u = t[s];
            if (u == v) continue;
            ax = __fadd_rn(ax, vin[3LL * u]);
            ay = __fadd_rn(ay, vin[3LL * u + 1]);
            az = __fadd_rn(az, vin[3LL * u + 2]);
            count++;
        }
    }
    const float inv = (float)(1.0 / (double)(float)count);   // vec3 operator/= (vmath.cpp:105-111)
    ax = __fmul_rn(ax, inv);
    ay = __fmul_rn(ay, inv);
    az = __fmul_rn(az, inv);
    const float x = vin[3LL * v], y = vin[3LL * v + 1], z = vin[3LL * v + 2];
    vout[3LL * v] = __fadd_rn(x, __fmul_rn(value, __fsub_rn(ax, x)));
    vout[3LL * v + 1] = __fadd_rn(y, __fmul_rn(value, __fsub_rn(ay, y)));
    vout[3LL * v + 2] = __fadd_rn(z, __fmul_rn(value, __fsub_rn(az, z)));
}

// ------------------------------------------------------------------ scans
// Exclusive scan of n int2 values into out[0..n] (out[n] = the totals), by
// tiles of TILE: tile sums, their scan in one CTA, then each tile again.
__global__ void __launch_bounds__(MESH_TPB) k_scan2_tiles(const int2 *in, long long n, int2 *tileSums) {
    const long long base = (long long)blockIdx.x * TILE + (long long)threadIdx.x * CELLS_PER_THREAD;
    int2 own = make_int2(0, 0);
    for (int q = 0; q < CELLS_PER_THREAD; q++)
        if (base + q < n) {
            own.x += in[base + q].x;
            own.y += in[base + q].y;
        }
    int2 tot;
    block_scan_int2(own, &tot);
    if (threadIdx.x == 0) tileSums[blockIdx.x] = tot;
}
__global__ void __launch_bounds__(MESH_TPB) k_scan2_apply(const int2 *in, long long n, const int2 *tileBase,
                                                          const int *totals, int2 *out) {
    const long long base = (long long)blockIdx.x * TILE + (long long)threadIdx.x * CELLS_PER_THREAD;
    int2 own = make_int2(0, 0);
    for (int q = 0; q < CELLS_PER_THREAD; q++)
        if (base + q < n) {
            own.x += in[base + q].x;
            own.y += in[base + q].y;
        }
    int2 tot;
    int2 run = block_scan_int2(own, &tot);
    run.x += tileBase[blockIdx.x].x;
    run.y += tileBase[blockIdx.x].y;
    for (int q = 0; q < CELLS_PER_THREAD; q++) {
        const long long t = base + q;
        if (t >= n) break;
        const int2 v = in[t];
        out[t] = run;
        run.x += v.x;
        run.y += v.y;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = make_int2(totals[0], totals[1]);
}

template <class T>
int grow(MeshBuffers &mb, T **p, long long *cap, long long need) {
    if (need <= *cap && *p) return FLIP_OK;
    if (*p) {
        cudaFree(*p);
        mb.bytes -= (long long)sizeof(T) * *cap;
        *p = nullptr;
        *cap = 0;
    }
    const long long want = std::max<long long>(need + need / 4, 1);
    cudaError_t e = cudaMalloc((void **)p, (size_t)want * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return record_error(FLIP_E_NOMEM, std::string("surface mesh buffers: ") + cudaGetErrorString(e));
    }
    *cap = want;
    mb.bytes += (long long)sizeof(T) * want;
    return FLIP_OK;
}

#define MCK(call)                                                                                         \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess) return record_error(FLIP_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)
#define MRC(call)                  \
    do {                           \
        int rc_ = (call);          \
        if (rc_) return rc_;       \
    } while (0)

}  // namespace

void mesh_release(MeshBuffers &mb) {
    void *ptrs[] = {mb.occ, mb.active, mb.field, mb.cube, mb.vstart, mb.tstart, mb.tiles, mb.totals,
                    mb.verts[0], mb.verts[1], mb.tris, mb.adj, mb.adjStart, mb.adjCursor, mb.adjList};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    mb = MeshBuffers{};
}

int mesh_surface(const MeshJob &job, MeshBuffers &mb, cudaStream_t s) {
    const StepConsts &c = job.c;
    mb.nverts = mb.ntris = 0;
    mb.cur = 0;
    if (job.n <= 0) return FLIP_OK;   // no particles: an empty mesh (fluidsimulation.cpp:5047-5051)
    const int sd = job.subdivisions;
    MeshFrame m{};
    m.I = c.I;
    m.J = c.J;
    m.K = c.K;
    m.dx = c.dx;
    m.invdx = 1.0 / c.dx;
    m.subdx = c.dx / (double)sd;
    m.invsub = 1.0 / m.subdx;
    m.invsubf = (float)m.invsub;
    m.blockdx = MB * m.subdx;
    m.invBlock = 1.0 / m.blockdx;
    m.invBlockf = (float)m.invBlock;
    m.blockdxF = (float)(MB * m.subdx);
    m.invBlockF = 1.0 / (double)m.blockdxF;
    m.invBlockFf = (float)m.invBlockF;
    m.r = (float)job.radius;
    m.sr = 1.5f * m.r;   // _searchRadiusFactor * r (particlemesher.h:193)
    m.maxd = (float)(3.0 * job.radius);
    const int sI = c.I * sd + 1, sJ = c.J * sd + 1, sK = c.K * sd + 1;
    m.nbI = (sI + MB - 1) / MB;
    m.nbJ = (sJ + MB - 1) / MB;
    m.nbK = (sK + MB - 1) / MB;
    const long long nb = (long long)m.nbI * m.nbJ * m.nbK;

    // blocks that hold particles, feathered by one block
    MRC(grow(mb, &mb.occ, &mb.occCap, nb));
    MCK(cudaMemsetAsync(mb.occ, 0, nb, s));
    { FLIP_COUNT(1); k_mesh_occupancy<<<div_up(job.n, MESH_TPB), MESH_TPB, 0, s>>>(job.p, job.n, m, mb.occ); }
    std::vector<uint8_t> occ(nb), act(nb, 0);
    MCK(cudaMemcpyAsync(occ.data(), mb.occ, nb, cudaMemcpyDeviceToHost, s));
    FLIP_SYNC_COUNT();
    MCK(cudaStreamSynchronize(s));
    auto bidx = [&](int a, int b, int e) { return a + (long long)m.nbI * (b + (long long)m.nbJ * e); };
    for (int e = 0; e < m.nbK; e++)
        for (int b = 0; b < m.nbJ; b++)
            for (int a = 0; a < m.nbI; a++) {
                if (!occ[bidx(a, b, e)]) continue;
                for (int z = std::max(e - 1, 0); z <= std::min(e + 1, m.nbK - 1); z++)
                    for (int y = std::max(b - 1, 0); y <= std::min(b + 1, m.nbJ - 1); y++)
                        for (int x = std::max(a - 1, 0); x <= std::min(a + 1, m.nbI - 1); x++) act[bidx(x, y, z)] = 1;
            }
    // the one compute chunk (particlemesher.cpp:139-282)
    int lo[3] = {m.nbI, m.nbJ, m.nbK}, hi[3] = {0, 0, 0};
    const int nbd[3] = {m.nbI, m.nbJ, m.nbK};
    bool any = false;
    for (int e = 0; e < m.nbK; e++)
        for (int b = 0; b < m.nbJ; b++)
            for (int a = 0; a < m.nbI; a++)
                if (act[bidx(a, b, e)]) {
                    any = true;
                    const int g[3] = {a, b, e};
                    for (int d = 0; d < 3; d++) {
                        lo[d] = std::min(lo[d], g[d]);
                        hi[d] = std::max(hi[d], g[d] + 1);
                    }
                }
    if (!any) return FLIP_OK;
    int split = 0;
    if (m.nbJ > m.nbI) split = 1;
    if (m.nbK > nbd[split]) split = 2;
    for (int d = 0; d < 3; d++)
        if (d != split) {
            lo[d] = std::max(lo[d] - 1, 0);
            hi[d] = std::min(hi[d] + 1, nbd[d]);
        }
    const int sub[3] = {sI, sJ, sK};
    int gmin[3], gmax[3];
    for (int d = 0; d < 3; d++) {
        gmin[d] = MB * lo[d];
        gmax[d] = std::min(MB * hi[d], sub[d]);
    }
    m.ni = gmax[0] - gmin[0];
    m.nj = gmax[1] - gmin[1];
    m.nk = gmax[2] - gmin[2];
    m.cbI = hi[0] - lo[0];
    m.cbJ = hi[1] - lo[1];
    m.cbK = hi[2] - lo[2];
    m.offx = (float)((double)(float)gmin[0] * m.subdx);   // Grid3d::GridIndexToPosition
    m.offy = (float)((double)(float)gmin[1] * m.subdx);
    m.offz = (float)((double)(float)gmin[2] * m.subdx);
    // AABB(pmin, pmax).expand(2 (r + 1e-6)) (particlemesher.cpp:287-292, aabb.cpp:40-52, 122-128)
    {
        const float pmx = (float)((double)(float)gmax[0] * m.subdx), pmy = (float)((double)(float)gmax[1] * m.subdx),
                    pmz = (float)((double)(float)gmax[2] * m.subdx);
        const double v = 2.0f * (job.radius + (double)1e-6f), h = 0.5 * v;
        m.bbx = m.offx - (float)h;
        m.bby = m.offy - (float)h;
        m.bbz = m.offz - (float)h;
        m.bbw = ((double)pmx - (double)m.offx) + v;
        m.bbh = ((double)pmy - (double)m.offy) + v;
        m.bbd = ((double)pmz - (double)m.offz) + v;
    }
    // how ScalarField::setSolidSDF finds solid nodes (scalarfield.cpp:372-395)
    const float offLen = std::sqrt(m.offx * m.offx + m.offy * m.offy + m.offz * m.offz);
    if (m.ni == c.I + 1 && m.nj == c.J + 1 && m.nk == c.K + 1 && std::fabs(m.subdx - c.dx) < 1e-12)
        m.solidMode = 2;
    else if (std::fabs(2 * m.subdx - c.dx) < 1e-6 && offLen < 1e-6)
        m.solidMode = 1;
    else
        m.solidMode = 0;
    const double scale = 0.1 / m.subdx;   // _localdx / _subdx (particlemesher.cpp:40-52)
    m.scalef = (float)scale;
    m.invscalef = (float)(1.0 / scale);

    const long long ncb = (long long)m.cbI * m.cbJ * m.cbK;
    std::vector<uint8_t> cact(ncb);
    for (int e = 0; e < m.cbK; e++)
        for (int b = 0; b < m.cbJ; b++)
            for (int a = 0; a < m.cbI; a++)
                cact[a + (long long)m.cbI * (b + (long long)m.cbJ * e)] = act[bidx(a + lo[0], b + lo[1], e + lo[2])];
    const long long nnodes = (long long)m.ni * m.nj * m.nk;
    const long long ncells = (long long)(m.ni - 1) * (m.nj - 1) * (m.nk - 1);
    const long long ntiles = std::max<long long>((ncells + TILE - 1) / TILE, 1);
    MRC(grow(mb, &mb.active, &mb.activeCap, ncb));
    MRC(grow(mb, &mb.field, &mb.fieldCap, nnodes));
    MRC(grow(mb, &mb.cube, &mb.cubeCap, std::max<long long>(ncells, 1)));
    MRC(grow(mb, &mb.vstart, &mb.vstartCap, std::max<long long>(ncells, 1)));
    MRC(grow(mb, &mb.tstart, &mb.tstartCap, std::max<long long>(ncells, 1)));
    MRC(grow(mb, &mb.tiles, &mb.tilesCap, ntiles));
    MRC(grow(mb, &mb.totals, &mb.totalsCap, 2));
    MCK(cudaMemcpyAsync(mb.active, cact.data(), ncb, cudaMemcpyHostToDevice, s));
    {
        dim3 grid(m.cbI, m.cbJ, m.cbK);
        FLIP_COUNT(1);
        k_mesh_field<<<grid, MESH_TPB, 0, s>>>(job.p, job.cellStart, m, mb.active, job.solidPhi, mb.field);
    }
    if (ncells <= 0) return FLIP_OK;
    { FLIP_COUNT(1); k_mesh_count<<<(unsigned)ntiles, MESH_TPB, 0, s>>>(m, mb.field, ncells, mb.cube, mb.tiles); }
    { FLIP_COUNT(1); k_mesh_scan_tiles<<<1, MESH_TPB, 0, s>>>(mb.tiles, (int)ntiles, mb.totals); }
    int totals[2];
    MCK(cudaMemcpyAsync(totals, mb.totals, sizeof(totals), cudaMemcpyDeviceToHost, s));
    FLIP_SYNC_COUNT();
    MCK(cudaStreamSynchronize(s));
    const int nverts = totals[0], ntris = totals[1];
    if (nverts <= 0 || ntris <= 0) return FLIP_OK;
    MRC(grow(mb, &mb.verts[0], &mb.vertsCap[0], 3LL * nverts));
    MRC(grow(mb, &mb.verts[1], &mb.vertsCap[1], 3LL * nverts));
    MRC(grow(mb, &mb.tris, &mb.trisCap, 3LL * ntris));
    {
        FLIP_COUNT(1);
        k_mesh_vertices<<<(unsigned)ntiles, MESH_TPB, 0, s>>>(m, mb.field, job.solidPhi, ncells, mb.cube, mb.tiles,
                                                               mb.vstart, mb.tstart, mb.verts[0]);
    }
    { FLIP_COUNT(1); k_mesh_triangles<<<div_up(ncells, MESH_TPB), MESH_TPB, 0, s>>>(m, ncells, mb.cube, mb.vstart, mb.tstart, mb.tris); }
    mb.nverts = nverts;
    mb.ntris = ntris;
    if (job.smoothIterations > 0) {
        // TriangleMesh::smooth (trianglemesh.cpp:572-583)
        const long long vt = (nverts + TILE - 1) / TILE;
        MRC(grow(mb, &mb.adj, &mb.adjCap, (long long)nverts));
        MRC(grow(mb, &mb.adjStart, &mb.adjStartCap, (long long)nverts + 1));
        MRC(grow(mb, &mb.adjCursor, &mb.adjCursorCap, (long long)nverts));
        MRC(grow(mb, &mb.adjList, &mb.adjListCap, 3LL * ntris));
        MRC(grow(mb, &mb.tiles, &mb.tilesCap, std::max(ntiles, vt)));
        MCK(cudaMemsetAsync(mb.adj, 0, (size_t)nverts * sizeof(int2), s));
        MCK(cudaMemsetAsync(mb.adjCursor, 0, (size_t)nverts * sizeof(int), s));
        { FLIP_COUNT(1); k_mesh_adj_count<<<div_up(3LL * ntris, MESH_TPB), MESH_TPB, 0, s>>>(mb.tris, ntris, mb.adj); }
        { FLIP_COUNT(1); k_scan2_tiles<<<(unsigned)vt, MESH_TPB, 0, s>>>(mb.adj, nverts, mb.tiles); }
        { FLIP_COUNT(1); k_mesh_scan_tiles<<<1, MESH_TPB, 0, s>>>(mb.tiles, (int)vt, mb.totals); }
        { FLIP_COUNT(1); k_scan2_apply<<<(unsigned)vt, MESH_TPB, 0, s>>>(mb.adj, nverts, mb.tiles, mb.totals, mb.adjStart); }
        { FLIP_COUNT(1); k_mesh_adj_fill<<<div_up(3LL * ntris, MESH_TPB), MESH_TPB, 0, s>>>(mb.tris, ntris, mb.adjStart, mb.adjCursor, mb.adjList); }
        { FLIP_COUNT(1); k_mesh_adj_sort<<<div_up(nverts, MESH_TPB), MESH_TPB, 0, s>>>(mb.adjStart, nverts, mb.adjList); }
        const float value = (float)job.smoothValue;
        for (int it = 0; it < job.smoothIterations; it++) {
            FLIP_COUNT(1);
            k_mesh_smooth<<<div_up(nverts, MESH_TPB), MESH_TPB, 0, s>>>(mb.verts[mb.cur], mb.verts[mb.cur ^ 1], mb.tris,
                                                                       mb.adjStart, mb.adjList, nverts, value);
            mb.cur ^= 1;
        }
    }
    MCK(cudaGetLastError());
    return FLIP_OK;
}

}  // namespace flip
