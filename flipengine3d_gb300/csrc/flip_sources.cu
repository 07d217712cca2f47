// Mesh fluid sources (addMeshFluidSource, fluidsimulation.cpp:1953-1992):
// the two per-substep passes that are not seeding.  Emission reuses the
// seeding kernels of flip_seed.cu with the source's level set, and the
// particle-velocity constraint runs inside the advection kernel.
//
//   * Inflow sources that constrain the fluid velocity keep the body force
//     off the P2G-valid faces where their level set is negative
//     (_getInflowConstrainedVelocityComponents, :3372-3440).  The reference
//     reads the level set at the face's world position without subtracting
//     the level set's offset, that is, in the level set's own frame; that is
//     kept, so the faces are the reference's.
//   * Outflow sources remove the particles in their cells (or, inversed,
//     outside them) where their level set at p - offset is negative
//     (non-negative, inversed) (_updateOutflowMeshFluidSource, :4608-4650).
#include "flip_device.cuh"

namespace flip {
namespace {

constexpr int TPB = 256;

__global__ void k_inflow_faces(StepConsts c, InflowConstraint ic, const uint8_t *vu, const uint8_t *vv,
                               const uint8_t *vw, uint8_t *ex) {
    const long long nu = (long long)(c.I + 1) * c.J * c.K, nv = (long long)c.I * (c.J + 1) * c.K,
                    nw = (long long)c.I * c.J * (c.K + 1);
    const long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nu + nv + nw) return;
    int dir, i, j, k;
    uint8_t valid;
    if (f < nu) {
        dir = 0;
        unflatten(f, c.I + 1, c.J, i, j, k);
        valid = vu[f];
    } else if (f < nu + nv) {
        dir = 1;
        unflatten(f - nu, c.I, c.J + 1, i, j, k);
        valid = vv[f - nu];
    } else {
        dir = 2;
        unflatten(f - nu - nv, c.I, c.J, i, j, k);
        valid = vw[f - nu - nv];
    }
    uint8_t out = 0;
    if (valid) {
        // Grid3d::FaceIndexToPositionU/V/W (grid3d.h:111-133)
        const float px = dir == 0 ? (float)((double)(float)i * c.dx) : (float)(((double)(float)i + 0.5) * c.dx);
        const float py = dir == 1 ? (float)((double)(float)j * c.dx) : (float)(((double)(float)j + 0.5) * c.dx);
        const float pz = dir == 2 ? (float)((double)(float)k * c.dx) : (float)(((double)(float)k + 0.5) * c.dx);
        for (int q = 0; q < ic.count && !out; q++)
            if (source_phi(ic.g[q], px, py, pz) < 0.0f) out = 1;
    }
    ex[f] = out;
}

__global__ void k_outflow_mark(ParticleSoA p, int n, StepConsts c, const uint8_t *cellMask, int inversed,
                               SourceGridView g, unsigned int *keys) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const float px = p.px[t], py = p.py[t], pz = p.pz[t];
    const int i = exact_floor(px, c.invdx, c.invdxf), j = exact_floor(py, c.invdx, c.invdxf),
              k = exact_floor(pz, c.invdx, c.invdxf);
    const Dims d{c.I, c.J, c.K};
    if (!d.in(i, j, k)) return;
    const bool listed = cellMask[d.idx(i, j, k)] != 0;
    if (inversed ? listed : !listed) return;
    const float v = source_phi(g, __fsub_rn(px, g.ox), __fsub_rn(py, g.oy), __fsub_rn(pz, g.oz));
    if (inversed ? v >= 0.0f : v < 0.0f) keys[t] |= KEY_SOLID;
}

}  // namespace

void launch_inflow_faces(const StepConsts &c, const InflowConstraint &ic, const uint8_t *vu, const uint8_t *vv,
                         const uint8_t *vw, uint8_t *ex, cudaStream_t s) {
    const long long tot = (long long)(c.I + 1) * c.J * c.K + (long long)c.I * (c.J + 1) * c.K +
                          (long long)c.I * c.J * (c.K + 1);
    FLIP_COUNT(1);
    k_inflow_faces<<<div_up(tot, TPB), TPB, 0, s>>>(c, ic, vu, vv, vw, ex);
}

void launch_outflow_mark(const ParticleSoA &p, int n, const StepConsts &c, const uint8_t *cellMask, int inversed,
                         const SourceGridView &g, unsigned int *keys, cudaStream_t s) {
    if (n <= 0) return;
    FLIP_COUNT(1);
    k_outflow_mark<<<div_up(n, TPB), TPB, 0, s>>>(p, n, c, cellMask, inversed, g, keys);
}

}  // namespace flip
