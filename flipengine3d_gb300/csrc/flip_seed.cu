// Seeding marker particles from a fluid mesh (addMeshFluid), on the device.
//
// The reference fills a queued fluid mesh at the end of the substep after it
// was added (_updateFluidObjects -> _updateAddedFluidMeshObjectQueue,
// fluidsimulation.cpp:4724-4759, 4794-4806): every cell around a grid node
// inside the mesh gets up to eight particles at the centres of its eight
// sub-cells (_addNewFluidCellsThread, :4522-4562).  A candidate is kept when
// the mesh's level set at it is <= 0; it is jittered when it lies deeper than
// one cell (or surface jitter is on); it must then sit in the fluid side of
// the solid level set, in the grid, and in a sub-cell that no particle holds
// yet (ParticleMaskGrid, particlemaskgrid.cpp:52-105; _addNewFluidCells,
// :4397-4430).  Particles are appended in cell order, then sub-cell order.
//
// Here one thread takes one candidate.  The order-dependent part, "a
// sub-cell is taken by the first candidate to reach it", becomes an atomic
// minimum of candidate indices per sub-cell, so the kept set is the
// reference's whatever the thread schedule; a scan of the keep flags gives
// each kept particle its place and its id.  Level-set values are evaluated in
// FP64 as the reference does (Interpolation::trilinearInterpolate,
// interpolation.cpp:72-113), since seeding runs once per added mesh.
//
// Jitter.  The reference draws it from the C library's rand(), from several
// threads at once, so its values are not reproducible.  Here candidate q's
// offset on axis a is a counter-based hash of (seed, q, a) mapped to [0, 1)
// and scaled as _randomDouble does (fluidsimulation.h:1501-1503): with the
// jitter factor at 0.001 the offset is exactly zero and the particles are
// the reference's bit for bit.
#include "flip_device.cuh"

namespace flip {

namespace {

constexpr int TPB = 256;

__device__ __forceinline__ int floor_div(float p, double inv) { return (int)floor((double)p * inv); }

// Interpolation::trilinearInterpolate over a nodal grid of (I+1)(J+1)(K+1)
// values, in the reference's FP64 arithmetic; out-of-grid corners read 0.
__device__ double nodal_at(const float *G, int I, int J, int K, double dx, float px, float py, float pz) {
    const double inv = 1.0 / dx;
    const int i = floor_div(px, inv), j = floor_div(py, inv), k = floor_div(pz, inv);
    const float gx = (float)((double)(float)i * dx), gy = (float)((double)(float)j * dx), gz = (float)((double)(float)k * dx);
    const double ix = (double)(px - gx) * inv, iy = (double)(py - gy) * inv, iz = (double)(pz - gz) * inv;
    const int ni = I + 1, nj = J + 1, nk = K + 1;
    auto at = [&](int a, int b, int c) -> double {
        const bool in = a >= 0 && b >= 0 && c >= 0 && a < ni && b < nj && c < nk;
        return in ? (double)G[(long long)a + (long long)ni * ((long long)b + (long long)nj * c)] : 0.0;
    };
    const double p0 = at(i, j, k), p1 = at(i + 1, j, k), p2 = at(i, j + 1, k), p3 = at(i, j, k + 1);
    const double p4 = at(i + 1, j, k + 1), p5 = at(i, j + 1, k + 1), p6 = at(i + 1, j + 1, k), p7 = at(i + 1, j + 1, k + 1);
    return p0 * (1 - ix) * (1 - iy) * (1 - iz) + p1 * ix * (1 - iy) * (1 - iz) + p2 * (1 - ix) * iy * (1 - iz) +
           p3 * (1 - ix) * (1 - iy) * iz + p4 * ix * (1 - iy) * iz + p5 * (1 - ix) * iy * iz +
           p6 * ix * iy * (1 - iz) + p7 * ix * iy * iz;
}

// SplitMix64's finaliser (Steele, Lea, Flood 2014) over a packed counter.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double uniform01(unsigned long long seed, long long q, int axis) {
    const unsigned long long h = mix64(seed + 0x9e3779b97f4a7c15ull * (unsigned long long)(3 * q + axis + 1));
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

// Sub-cell of a point (ParticleMaskGrid: positions at dx / 2) and its bit in
// the cell's 8-bit mask, packed four cells to a 32-bit word.
struct SubCell {
    long long cell;      // flat cell index
    long long sub;       // flat sub-cell index over 2I x 2J x 2K
    unsigned int bit;    // bit within the cell's word
    bool in;
};
__device__ __forceinline__ SubCell sub_cell(const StepConsts &c, float px, float py, float pz) {
    const double inv2 = 1.0 / (0.5 * c.dx);
    const int si = floor_div(px, inv2), sj = floor_div(py, inv2), sk = floor_div(pz, inv2);
    SubCell s;
    s.in = si >= 0 && sj >= 0 && sk >= 0 && si < 2 * c.I && sj < 2 * c.J && sk < 2 * c.K;
    const int ci = si >> 1, cj = sj >> 1, ck = sk >> 1;
    s.cell = (long long)ci + (long long)c.I * ((long long)cj + (long long)c.J * ck);
    s.sub = (long long)si + 2LL * c.I * ((long long)sj + 2LL * c.J * sk);
    const int mcase = (si & 1) | ((sj & 1) << 1) | ((sk & 1) << 2);
    s.bit = 1u << ((unsigned)(s.cell & 3) * 8u + (unsigned)mcase);
    return s;
}

__global__ void k_mask_particles(ParticleSoA p, int n, StepConsts c, unsigned int *mask) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const SubCell s = sub_cell(c, p.px[t], p.py[t], p.pz[t]);
    if (s.in) atomicOr(&mask[s.cell >> 2], s.bit);
}

struct SeedArgs {
    const int *cells;       // flat cell indices, ascending
    long long ncand;        // 8 per cell
    SourceGridView mesh;    // nodal level set of the mesh and its first node's position
    const float *solidPhi;  // nodal solid level set
    double jitter;          // _getMarkerParticleJitter()
    int jitterSurface;      // _isJitterSurfaceMarkerParticlesEnabled
    unsigned long long seed;
};

// Candidate q = 8 * cell + sub-cell offset: its position after the tests, or
// no claim.  A passing candidate claims its sub-cell with an atomic minimum.
__global__ void k_seed_candidates(StepConsts c, SeedArgs a, const unsigned int *mask, float4 *cand,
                                  unsigned int *owner) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= a.ncand) return;
    const int cell = a.cells[q >> 3], o = (int)(q & 7);
    int i, j, k;
    unflatten(cell, c.I, c.J, i, j, k);
    // cell centre plus the sub-cell offset (vec3 of +-0.25 dx, in float)
    const float qo = (float)(0.25 * c.dx);
    const float ox = (o & 1) ? qo : -qo, oy = (o & 2) ? qo : -qo, oz = (o & 4) ? qo : -qo;
    float px = __fadd_rn(cell_centre(i, c.dx), ox), py = __fadd_rn(cell_centre(j, c.dx), oy),
          pz = __fadd_rn(cell_centre(k, c.dx), oz);
    cand[q] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    // meshSDF.trilinearInterpolate(p - sdfoffset), a float (fluidsimulation.cpp:4548)
    const double d = (double)source_phi(a.mesh, __fsub_rn(px, a.mesh.ox), __fsub_rn(py, a.mesh.oy),
                                        __fsub_rn(pz, a.mesh.oz));
    if (d > 0) return;
    if (a.jitterSurface || d < -c.dx) {
        const double lo = -a.jitter, hi = a.jitter;
        px = (float)((double)px + (lo + uniform01(a.seed, q, 0) * (hi - lo)));
        py = (float)((double)py + (lo + uniform01(a.seed, q, 1) * (hi - lo)));
        pz = (float)((double)pz + (lo + uniform01(a.seed, q, 2) * (hi - lo)));
    }
    if (!((float)nodal_at(a.solidPhi, c.I, c.J, c.K, c.dx, px, py, pz) > 0)) return;
    const SubCell s = sub_cell(c, px, py, pz);
    if (!s.in) return;   // _addMarkerParticle keeps points whose cell is in the grid
    if (mask[s.cell >> 2] & s.bit) return;
    cand[q] = make_float4(px, py, pz, 1.0f);
    atomicMin(&owner[s.sub], (unsigned int)q);
}

__global__ void k_seed_keep(StepConsts c, long long ncand, const float4 *cand, const unsigned int *owner, int *keep) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= ncand) return;
    const float4 p = cand[q];
    bool k = false;
    if (p.w != 0.0f) k = owner[sub_cell(c, p.x, p.y, p.z).sub] == (unsigned int)q;
    keep[q] = k ? 1 : 0;
}

__global__ void k_seed_scatter(StepConsts c, long long ncand, const float4 *cand, const int *keep, const int *rank,
                               ParticleSoA p, int n0, unsigned int id0, float vx, float vy, float vz,
                               unsigned int *mask) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= ncand || !keep[q]) return;
    const float4 v = cand[q];
    const int d = n0 + rank[q];
    p.px[d] = v.x; p.py[d] = v.y; p.pz[d] = v.z;
    p.vx[d] = vx; p.vy[d] = vy; p.vz[d] = vz;
    p.id[d] = id0 + (unsigned int)rank[q];
    const SubCell s = sub_cell(c, v.x, v.y, v.z);
    atomicOr(&mask[s.cell >> 2], s.bit);
}

}  // namespace

void launch_mask_particles(const ParticleSoA &p, int n, const StepConsts &c, unsigned int *mask, cudaStream_t s) {
    if (n <= 0) return;
    FLIP_COUNT(1);
    k_mask_particles<<<div_up(n, TPB), TPB, 0, s>>>(p, n, c, mask);
}

void launch_seed_candidates(const StepConsts &c, const int *cells, long long ncells, const SourceGridView &meshPhi,
                            const float *solidPhi, double jitter, bool jitterSurface, unsigned long long seed,
                            const unsigned int *mask, float4 *cand, unsigned int *owner, int *keep, cudaStream_t s) {
    if (ncells <= 0) return;
    SeedArgs a;
    a.cells = cells; a.ncand = 8 * ncells; a.mesh = meshPhi; a.solidPhi = solidPhi;
    a.jitter = jitter; a.jitterSurface = jitterSurface ? 1 : 0; a.seed = seed;
    const long long nb = div_up(a.ncand, TPB);
    { FLIP_COUNT(1); k_seed_candidates<<<(unsigned)nb, TPB, 0, s>>>(c, a, mask, cand, owner); }
    { FLIP_COUNT(1); k_seed_keep<<<(unsigned)nb, TPB, 0, s>>>(c, a.ncand, cand, owner, keep); }
}

void launch_seed_scatter(const StepConsts &c, long long ncand, const float4 *cand, const int *keep, const int *rank,
                         const ParticleSoA &p, int n0, unsigned int id0, float vx, float vy, float vz,
                         unsigned int *mask, cudaStream_t s) {
    if (ncand <= 0) return;
    FLIP_COUNT(1);
    k_seed_scatter<<<(unsigned)div_up(ncand, TPB), TPB, 0, s>>>(c, ncand, cand, keep, rank, p, n0, id0, vx, vy, vz,
                                                                mask);
}

}  // namespace flip
