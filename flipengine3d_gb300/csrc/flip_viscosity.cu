// Viscosity (setViscosity; _applyViscosityToVelocityField,
// fluidsimulation.cpp:3592-3640): Batty's variational viscosity as the
// reference's ViscositySolver sets it up (viscositysolver.cpp:49-891),
// solved on the GPU.
//
// The set-up follows the reference operation by operation: face states from
// the solid level set at cell centres (:97-202), liquid cells dilated by two
// layers (:204-238), the liquid volume fractions of the cell, face and edge
// control volumes from the liquid level set at the control volumes' corners
// (:240-368, LevelsetUtils::volumeFraction), the faces in the system
// (:374-464) and each row's coefficients and right-hand side (:466-821).
// A corner value is sampled once, by the first valid control volume in flat
// order that touches it, at that volume's centre plus the corner's offset,
// as the reference's nodal cache does, so the fractions are the reference's
// bit for bit.
//
// The solve differs on purpose.  The reference runs its FP32 MIC(0)-PCG to
// a relative residual of 1e-4 (at most 700 iterations).  Here the system is
// solved matrix-free by Jacobi-preconditioned CG in FP64 to 1e-9, so the
// result is the system's solution to well inside the reference's own
// tolerance; a reference-exact MIC(0) over this 15-point, three-component
// system would be a sequential triangular solve.  The faces of the system
// then take the solution and every other face is zeroed, as the reference's
// _applySolutionToVelocityField (:856-891) does.
#include <cmath>
#include <string>

#include "../../include/flip3d.h"
#include "flip_device.cuh"

namespace flip {
namespace {

constexpr int TPB = 256;

// ---------------------------------------------------------------- geometry
struct VGrid {   // one control-volume grid: extents and corner offset from the cell centre
    int ni, nj, nk;
    float ox, oy, oz;
};

// LevelsetUtils::volumeFraction (levelsetutils.cpp:213-260, levelsetutils.h:62-104), float
__device__ __forceinline__ void sort4(float &a, float &b, float &c, float &d) {
    float t;
    if (a > b) { t = a; a = b; b = t; }
    if (c > d) { t = c; c = d; d = t; }
    if (a > c) { t = a; a = c; c = t; }
    if (b > d) { t = b; b = d; d = t; }
    if (b > c) { t = b; b = c; c = t; }
}
__device__ __forceinline__ float tet_fraction(float p0, float p1, float p2, float p3) {
    return __fdiv_rn(__fmul_rn(__fmul_rn(p0, p0), p0),
                     __fmul_rn(__fmul_rn(__fsub_rn(p0, p1), __fsub_rn(p0, p2)), __fsub_rn(p0, p3)));
}
__device__ __forceinline__ float prism_fraction(float p0, float p1, float p2, float p3) {
    const float a = __fdiv_rn(p0, __fsub_rn(p0, p2));
    const float b = __fdiv_rn(p0, __fsub_rn(p0, p3));
    const float c = __fdiv_rn(p1, __fsub_rn(p1, p3));
    const float d = __fdiv_rn(p1, __fsub_rn(p1, p2));
    return __fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(a, b), __fsub_rn(1.0f, d)),
                               __fmul_rn(__fmul_rn(b, __fsub_rn(1.0f, c)), d)),
                     __fmul_rn(c, d));
}
__device__ float tet_volume(float p0, float p1, float p2, float p3) {
    sort4(p0, p1, p2, p3);
    if (p3 <= 0) return 1.0f;
    if (p2 <= 0) return __fsub_rn(1.0f, tet_fraction(p3, p2, p1, p0));
    if (p1 <= 0) return prism_fraction(p0, p1, p2, p3);
    if (p0 <= 0) return tet_fraction(p0, p1, p2, p3);
    return 0.0f;
}
__device__ float cube_volume(float p000, float p100, float p010, float p110, float p001, float p101, float p011,
                             float p111) {
    float s = tet_volume(p000, p001, p101, p011);
    s = __fadd_rn(s, tet_volume(p000, p101, p100, p110));
    s = __fadd_rn(s, tet_volume(p000, p010, p011, p110));
    s = __fadd_rn(s, tet_volume(p101, p011, p111, p110));
    s = __fadd_rn(s, __fmul_rn(2.0f, tet_volume(p000, p011, p101, p110)));
    s = __fadd_rn(s, tet_volume(p100, p101, p001, p111));
    s = __fadd_rn(s, tet_volume(p100, p001, p000, p010));
    s = __fadd_rn(s, tet_volume(p100, p110, p111, p010));
    s = __fadd_rn(s, tet_volume(p001, p111, p011, p010));
    s = __fadd_rn(s, __fmul_rn(2.0f, tet_volume(p100, p111, p001, p010)));
    return __fdiv_rn(s, 12.0f);
}

// ParticleLevelSet::trilinearInterpolate (particlelevelset.cpp:136-138): the
// cell-centred liquid level set, read at p - dx/2 as a nodal grid, FP64
// weights, corners outside the grid 0, rounded to float.
__device__ float liquid_at(const StepConsts &c, const float *phi, float px, float py, float pz) {
    const float h = (float)(0.5 * c.dx);
    SourceGridView g{phi, c.I, c.J, c.K, 0.0f, 0.0f, 0.0f, c.dx};
    return source_phi(g, __fsub_rn(px, h), __fsub_rn(py, h), __fsub_rn(pz, h));
}

// ------------------------------------------------------------------ states
// Face states (viscositysolver.cpp:135-202): solid on the domain's border
// faces and where the solid level set's cell-centre values on the face's two
// sides sum to <= 0; cell-centre value = the mean of the cell's 8 nodes
// (MeshLevelSet::getDistanceAtCellCenter, meshlevelset.cpp:151-162).
__device__ __forceinline__ float solid_centre(const StepConsts &c, const float *S, int i, int j, int k) {
    const int ni = c.I + 1, nj = c.J + 1;
    auto at = [&](int a, int b, int d) { return S[(long long)a + (long long)ni * ((long long)b + (long long)nj * d)]; };
    float s = at(i, j, k);
    s = __fadd_rn(s, at(i + 1, j, k));
    s = __fadd_rn(s, at(i, j + 1, k));
    s = __fadd_rn(s, at(i + 1, j + 1, k));
    s = __fadd_rn(s, at(i, j, k + 1));
    s = __fadd_rn(s, at(i + 1, j, k + 1));
    s = __fadd_rn(s, at(i, j + 1, k + 1));
    s = __fadd_rn(s, at(i + 1, j + 1, k + 1));
    return __fmul_rn(0.125f, s);
}
__global__ void k_visc_states(StepConsts c, const float *S, uint8_t *fluidFace) {
    const long long nu = (long long)(c.I + 1) * c.J * c.K, nv = (long long)c.I * (c.J + 1) * c.K,
                    nw = (long long)c.I * c.J * (c.K + 1);
    const long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nu + nv + nw) return;
    int i, j, k;
    bool fluid;
    if (f < nu) {
        unflatten(f, c.I + 1, c.J, i, j, k);
        fluid = !(i == 0 || i == c.I) &&
                __fadd_rn(solid_centre(c, S, i - 1, j, k), solid_centre(c, S, i, j, k)) > 0.0f;
    } else if (f < nu + nv) {
        unflatten(f - nu, c.I, c.J + 1, i, j, k);
        fluid = !(j == 0 || j == c.J) &&
                __fadd_rn(solid_centre(c, S, i, j - 1, k), solid_centre(c, S, i, j, k)) > 0.0f;
    } else {
        unflatten(f - nu - nv, c.I, c.J, i, j, k);
        fluid = !(k == 0 || k == c.K) &&
                __fadd_rn(solid_centre(c, S, i, j, k - 1), solid_centre(c, S, i, j, k)) > 0.0f;
    }
    fluidFace[f] = fluid ? 1 : 0;
}

// Valid control volumes (viscositysolver.cpp:207-238): cells with liquid
// phi < 0 on an (I+1)(J+1)(K+1) grid, dilated twice over 6 neighbours.
__global__ void k_visc_valid(StepConsts c, const float *phi, uint8_t *valid) {
    const long long n = (long long)(c.I + 1) * (c.J + 1) * (c.K + 1);
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int i, j, k;
    unflatten(t, c.I + 1, c.J + 1, i, j, k);
    valid[t] = (i < c.I && j < c.J && k < c.K && phi[(long long)i + (long long)c.I * ((long long)j + (long long)c.J * k)] < 0.0f)
                   ? 1 : 0;
}
__global__ void k_visc_dilate(StepConsts c, const uint8_t *in, uint8_t *out) {
    const int ni = c.I + 1, nj = c.J + 1, nk = c.K + 1;
    const long long n = (long long)ni * nj * nk;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int i, j, k;
    unflatten(t, ni, nj, i, j, k);
    auto v = [&](int a, int b, int d) {
        return a >= 0 && b >= 0 && d >= 0 && a < ni && b < nj && d < nk &&
               in[(long long)a + (long long)ni * ((long long)b + (long long)nj * d)];
    };
    out[t] = (v(i, j, k) || v(i - 1, j, k) || v(i + 1, j, k) || v(i, j - 1, k) || v(i, j + 1, k) || v(i, j, k - 1) ||
              v(i, j, k + 1)) ? 1 : 0;
}

// Corner values of one control-volume grid (viscositysolver.cpp:278-368):
// node (a, b, d) of the grid's (ni+1)(nj+1)(nk+1) corners takes its value
// from the first valid volume in flat order among the eight that share it,
// sampled at that volume's centre plus the corner's offset.
__global__ void k_visc_corners(StepConsts c, VGrid g, const uint8_t *valid, const float *phi, float *node) {
    const int ni = g.ni + 1, nj = g.nj + 1, nk = g.nk + 1;
    const long long n = (long long)ni * nj * nk;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int a, b, d;
    unflatten(t, ni, nj, a, b, d);
    const int vi = c.I + 1, vj = c.J + 1;
    float val = 0.0f;
    // cells in ascending flat order: lower k first, then lower j, then lower i
    for (int q = 0; q < 8; q++) {
        const int dz = (q >> 2) & 1, dy = (q >> 1) & 1, dxx = q & 1;
        const int ci = a - 1 + dxx, cj = b - 1 + dy, ck = d - 1 + dz;
        if (ci < 0 || cj < 0 || ck < 0 || ci >= g.ni || cj >= g.nj || ck >= g.nk) continue;
        if (!valid[(long long)ci + (long long)vi * ((long long)cj + (long long)vj * ck)]) continue;
        // centre = centerStart + GridIndexToCellCenter(ci, cj, ck, dx), then +-dx/2
        const float hdx = __fmul_rn(0.5f, (float)c.dx);
        const float cx = __fadd_rn(g.ox, (float)((double)(float)ci * c.dx + 0.5 * c.dx));
        const float cy = __fadd_rn(g.oy, (float)((double)(float)cj * c.dx + 0.5 * c.dx));
        const float cz = __fadd_rn(g.oz, (float)((double)(float)ck * c.dx + 0.5 * c.dx));
        // node (a, b, d) is corner (1 - dxx, 1 - dy, 1 - dz) of this cell
        const float px = __fadd_rn(cx, dxx ? -hdx : hdx);
        const float py = __fadd_rn(cy, dy ? -hdx : hdx);
        const float pz = __fadd_rn(cz, dz ? -hdx : hdx);
        val = liquid_at(c, phi, px, py, pz);
        break;
    }
    node[t] = val;
}
__global__ void k_visc_volumes(StepConsts c, VGrid g, const uint8_t *valid, const float *node, float *vol) {
    const long long n = (long long)g.ni * g.nj * g.nk;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int i, j, k;
    unflatten(t, g.ni, g.nj, i, j, k);
    const int vi = c.I + 1, vj = c.J + 1;
    if (!valid[(long long)i + (long long)vi * ((long long)j + (long long)vj * k)]) {
        vol[t] = 0.0f;
        return;
    }
    const int ni = g.ni + 1, nj = g.nj + 1;
    auto nd = [&](int a, int b, int d) { return node[(long long)a + (long long)ni * ((long long)b + (long long)nj * d)]; };
    const float p000 = nd(i, j, k), p001 = nd(i, j, k + 1), p010 = nd(i, j + 1, k), p011 = nd(i, j + 1, k + 1);
    const float p100 = nd(i + 1, j, k), p101 = nd(i + 1, j, k + 1), p110 = nd(i + 1, j + 1, k),
                p111 = nd(i + 1, j + 1, k + 1);
    float v;
    if (p000 < 0 && p001 < 0 && p010 < 0 && p011 < 0 && p100 < 0 && p101 < 0 && p110 < 0 && p111 < 0) v = 1.0f;
    else if (p000 >= 0 && p001 >= 0 && p010 >= 0 && p011 >= 0 && p100 >= 0 && p101 >= 0 && p110 >= 0 && p111 >= 0)
        v = 0.0f;
    else v = cube_volume(p000, p100, p010, p110, p001, p101, p011, p111);
    vol[t] = v;
}

// ------------------------------------------------------------------ system
// The control-volume grids, in the order of ViscosityVolumeGrid
// (viscositysolver.h:57-78): centre, U, V, W, edgeU, edgeV, edgeW.
enum { VC = 0, VU, VV, VW, EU, EV, EW, NVOL };
struct VolPtrs {
    const float *v[NVOL];
    int ni[NVOL], nj[NVOL];
};
__device__ __forceinline__ float vol(const VolPtrs &p, int g, int i, int j, int k) {
    return p.v[g][(long long)i + (long long)p.ni[g] * ((long long)j + (long long)p.nj[g] * k)];
}
struct FaceIdx {   // flat index of a face over the U, V, W grids, one after the other
    int I, J, K;
    long long nu, nv;
    __device__ long long u(int i, int j, int k) const { return (long long)i + (long long)(I + 1) * ((long long)j + (long long)J * k); }
    __device__ long long v(int i, int j, int k) const { return nu + (long long)i + (long long)I * ((long long)j + (long long)(J + 1) * k); }
    __device__ long long w(int i, int j, int k) const { return nu + nv + (long long)i + (long long)I * ((long long)j + (long long)J * k); }
    __device__ long long of(int d, int i, int j, int k) const { return d == 0 ? u(i, j, k) : d == 1 ? v(i, j, k) : w(i, j, k); }
};
// One coupling of a row, in the order the reference adds them: the face
// (direction, offset), which of the six factors, and its sign.
struct Term { signed char d, di, dj, dk, f, s; };
enum { FR = 0, FL, FT, FB, FF, FK };
__constant__ Term kTerms[3][14] = {
    {{0, 1, 0, 0, FR, -1}, {0, -1, 0, 0, FL, -1}, {0, 0, 1, 0, FT, -1}, {0, 0, -1, 0, FB, -1}, {0, 0, 0, 1, FF, -1},
     {0, 0, 0, -1, FK, -1}, {1, 0, 1, 0, FT, -1}, {1, -1, 1, 0, FT, 1}, {1, 0, 0, 0, FB, 1}, {1, -1, 0, 0, FB, -1},
     {2, 0, 0, 1, FF, -1}, {2, -1, 0, 1, FF, 1}, {2, 0, 0, 0, FK, 1}, {2, -1, 0, 0, FK, -1}},
    {{1, 1, 0, 0, FR, -1}, {1, -1, 0, 0, FL, -1}, {1, 0, 1, 0, FT, -1}, {1, 0, -1, 0, FB, -1}, {1, 0, 0, 1, FF, -1},
     {1, 0, 0, -1, FK, -1}, {0, 1, 0, 0, FR, -1}, {0, 1, -1, 0, FR, 1}, {0, 0, 0, 0, FL, 1}, {0, 0, -1, 0, FL, -1},
     {2, 0, 0, 1, FF, -1}, {2, 0, -1, 1, FF, 1}, {2, 0, 0, 0, FK, 1}, {2, 0, -1, 0, FK, -1}},
    {{2, 1, 0, 0, FR, -1}, {2, -1, 0, 0, FL, -1}, {2, 0, 1, 0, FT, -1}, {2, 0, -1, 0, FB, -1}, {2, 0, 0, 1, FF, -1},
     {2, 0, 0, -1, FK, -1}, {0, 1, 0, 0, FR, -1}, {0, 1, 0, -1, FR, 1}, {0, 0, 0, 0, FL, 1}, {0, 0, 0, -1, FL, -1},
     {1, 0, 1, 0, FT, -1}, {1, 0, 1, -1, FT, 1}, {1, 0, 0, 0, FB, 1}, {1, 0, 0, -1, FB, -1}}};
// The control volume behind each factor of a row of direction d: (grid, di, dj, dk)
__constant__ signed char kVol[3][7][4] = {
    {{VU, 0, 0, 0}, {VC, 0, 0, 0}, {VC, -1, 0, 0}, {EW, 0, 1, 0}, {EW, 0, 0, 0}, {EV, 0, 0, 1}, {EV, 0, 0, 0}},
    {{VV, 0, 0, 0}, {EW, 1, 0, 0}, {EW, 0, 0, 0}, {VC, 0, 0, 0}, {VC, 0, -1, 0}, {EU, 0, 0, 1}, {EU, 0, 0, 0}},
    {{VW, 0, 0, 0}, {EV, 1, 0, 0}, {EV, 0, 0, 0}, {EU, 0, 1, 0}, {EU, 0, 0, 0}, {VC, 0, 0, 0}, {VC, 0, 0, -1}}};

struct SysArgs {
    FaceIdx fx;
    VolPtrs vp;
    const uint8_t *fluidFace;
    const float *u, *v, *w;
    float visc;     // the (constant) viscosity
    float factor;   // dt / dx^2 as the reference rounds it
};

// Per face: in the system or not (viscositysolver.cpp:374-464), its six
// factors, diagonal and right-hand side (:550-821), all in float.
__global__ void k_visc_rows(SysArgs a, uint8_t *inSys, float4 *fac, float4 *dr) {
    const long long nf = a.fx.nu + a.fx.nv + (long long)a.fx.I * a.fx.J * (a.fx.K + 1);
    const long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    int d, i, j, k;
    if (f < a.fx.nu) { d = 0; unflatten(f, a.fx.I + 1, a.fx.J, i, j, k); }
    else if (f < a.fx.nu + a.fx.nv) { d = 1; unflatten(f - a.fx.nu, a.fx.I, a.fx.J + 1, i, j, k); }
    else { d = 2; unflatten(f - a.fx.nu - a.fx.nv, a.fx.I, a.fx.J, i, j, k); }
    uint8_t in = 0;
    if (i >= 1 && j >= 1 && k >= 1 && i < a.fx.I && j < a.fx.J && k < a.fx.K && a.fluidFace[f]) {
        float vv[7];
#pragma unroll
        for (int q = 0; q < 7; q++)
            vv[q] = vol(a.vp, kVol[d][q][0], i + kVol[d][q][1], j + kVol[d][q][2], k + kVol[d][q][3]);
        in = (vv[0] > 0.0f || vv[1] > 0.0f || vv[2] > 0.0f || vv[3] > 0.0f || vv[4] > 0.0f || vv[5] > 0.0f ||
              vv[6] > 0.0f) ? 1 : 0;
        if (in) {
            const float v = a.visc;
            const float vq = __fmul_rn(0.25f, __fadd_rn(__fadd_rn(__fadd_rn(v, v), v), v));
            const float two = __fmul_rn(2.0f, a.factor);
            float F[6];
#pragma unroll
            for (int q = 0; q < 6; q++) {
                // the two factors across the row's own direction use the
                // viscosity at the cell centres, doubled; the others the
                // mean of four
                const bool own = (d == 0 && q < 2) || (d == 1 && (q == 2 || q == 3)) || (d == 2 && q >= 4);
                F[q] = own ? __fmul_rn(__fmul_rn(two, v), vv[q + 1]) : __fmul_rn(__fmul_rn(a.factor, vq), vv[q + 1]);
            }
            float diag = vv[0];
#pragma unroll
            for (int q = 0; q < 6; q++) diag = __fadd_rn(diag, F[q]);
            const float *G[3] = {a.u, a.v, a.w};
            const long long self = f - (d == 0 ? 0 : d == 1 ? a.fx.nu : a.fx.nu + a.fx.nv);
            float rval = __fmul_rn(vv[0], G[d][self]);
            for (int q = 0; q < 14; q++) {
                const Term t = kTerms[d][q];
                const long long g = a.fx.of(t.d, i + t.di, j + t.dj, k + t.dk);
                if (a.fluidFace[g]) continue;   // SOLID: the known velocity moves to the right-hand side
                const long long gl = g - (t.d == 0 ? 0 : t.d == 1 ? a.fx.nu : a.fx.nu + a.fx.nv);
                const float entry = t.s < 0 ? -F[t.f] : F[t.f];
                rval = __fsub_rn(rval, __fmul_rn(entry, G[t.d][gl]));
            }
            fac[2 * f] = make_float4(F[0], F[1], F[2], F[3]);
            fac[2 * f + 1] = make_float4(F[4], F[5], 0.0f, 0.0f);
            dr[f] = make_float4(diag, rval, 0.0f, 0.0f);
        }
    }
    inSys[f] = in;
}

// ------------------------------------------------------------------- solve
// Jacobi-preconditioned CG in FP64 over the faces in the system.  Reductions
// go through fixed per-block partials summed by one block, so they are
// deterministic.  scal: [0] r.z  [1] p.q  [2] new r.z  [3] |r|inf  [4] |b|inf
// [5] rows  [6] alpha  [7] beta
constexpr int RB = 1024;   // reduction blocks

__device__ __forceinline__ double block_sum(double v, double *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) s += sh[q];
    __syncthreads();
    return s;
}
__device__ __forceinline__ double block_max(double v, double *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) s = fmax(s, sh[q]);
    __syncthreads();
    return s;
}

struct CgArgs {
    SysArgs s;
    const uint8_t *inSys;
    const float4 *fac, *dr;
    long long nf;
    double *x, *r, *z, *p, *q;
    double *part;    // 3 x RB partials
    double *scal;
};

// A p for row f (zero off the system): diagonal plus the row's couplings to
// faces in the system, as the reference's matrix holds them.
__device__ double apply_row(const CgArgs &a, long long f) {
    int d, i, j, k;
    if (f < a.s.fx.nu) { d = 0; unflatten(f, a.s.fx.I + 1, a.s.fx.J, i, j, k); }
    else if (f < a.s.fx.nu + a.s.fx.nv) { d = 1; unflatten(f - a.s.fx.nu, a.s.fx.I, a.s.fx.J + 1, i, j, k); }
    else { d = 2; unflatten(f - a.s.fx.nu - a.s.fx.nv, a.s.fx.I, a.s.fx.J, i, j, k); }
    const float4 f0 = a.fac[2 * f], f1 = a.fac[2 * f + 1];
    const float F[6] = {f0.x, f0.y, f0.z, f0.w, f1.x, f1.y};
    double y = (double)a.dr[f].x * a.p[f];
    for (int q = 0; q < 14; q++) {
        const Term t = kTerms[d][q];
        const long long g = a.s.fx.of(t.d, i + t.di, j + t.dj, k + t.dk);
        if (!a.s.fluidFace[g] || !a.inSys[g]) continue;
        const double entry = t.s < 0 ? -(double)F[t.f] : (double)F[t.f];
        y += entry * a.p[g];
    }
    return y;
}

__global__ void k_cg_init(CgArgs a) {
    __shared__ double sh[32];
    double rz = 0.0, bmax = 0.0, rows = 0.0;
    for (long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x; f < a.nf; f += (long long)gridDim.x * blockDim.x) {
        double b = 0.0, z = 0.0;
        if (a.inSys[f]) {
            b = (double)a.dr[f].y;
            z = b / (double)a.dr[f].x;
            rz += b * z;
            bmax = fmax(bmax, fabs(b));
            rows += 1.0;
        }
        a.x[f] = 0.0;
        a.r[f] = b;
        a.z[f] = z;
        a.p[f] = z;
    }
    const double s0 = block_sum(rz, sh), s1 = block_max(bmax, sh), s2 = block_sum(rows, sh);
    if (threadIdx.x == 0) {
        a.part[blockIdx.x] = s0;
        a.part[RB + blockIdx.x] = s1;
        a.part[2 * RB + blockIdx.x] = s2;
    }
}
// mode 0: init sums -> rz, |b|, rows; 1: p.q; 2: new rz, |r| and beta
__global__ void k_cg_sum(CgArgs a, int mode) {
    __shared__ double sh[32];
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int q = threadIdx.x; q < RB; q += blockDim.x) {
        s0 += a.part[q];
        s1 = fmax(s1, a.part[RB + q]);
        s2 += a.part[2 * RB + q];
    }
    const double t0 = block_sum(s0, sh), t1 = block_max(s1, sh), t2 = block_sum(s2, sh);
    if (threadIdx.x != 0) return;
    if (mode == 0) { a.scal[0] = t0; a.scal[4] = t1; a.scal[3] = t1; a.scal[5] = t2; }
    else if (mode == 1) { a.scal[1] = t0; a.scal[6] = t0 != 0.0 ? a.scal[0] / t0 : 0.0; }
    else { a.scal[7] = a.scal[0] != 0.0 ? t0 / a.scal[0] : 0.0; a.scal[0] = t0; a.scal[3] = t1; }
}
__global__ void k_cg_apply(CgArgs a) {
    __shared__ double sh[32];
    double pq = 0.0;
    for (long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x; f < a.nf; f += (long long)gridDim.x * blockDim.x) {
        double y = 0.0;
        if (a.inSys[f]) {
            y = apply_row(a, f);
            pq += a.p[f] * y;
        }
        a.q[f] = y;
    }
    const double s0 = block_sum(pq, sh);
    if (threadIdx.x == 0) {
        a.part[blockIdx.x] = s0;
        a.part[RB + blockIdx.x] = 0.0;
        a.part[2 * RB + blockIdx.x] = 0.0;
    }
}
__global__ void k_cg_update(CgArgs a) {
    __shared__ double sh[32];
    const double alpha = a.scal[6];
    double rz = 0.0, rmax = 0.0;
    for (long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x; f < a.nf; f += (long long)gridDim.x * blockDim.x) {
        if (!a.inSys[f]) continue;
        a.x[f] += alpha * a.p[f];
        const double r = a.r[f] - alpha * a.q[f];
        a.r[f] = r;
        const double z = r / (double)a.dr[f].x;
        a.z[f] = z;
        rz += r * z;
        rmax = fmax(rmax, fabs(r));
    }
    const double s0 = block_sum(rz, sh), s1 = block_max(rmax, sh);
    if (threadIdx.x == 0) {
        a.part[blockIdx.x] = s0;
        a.part[RB + blockIdx.x] = s1;
        a.part[2 * RB + blockIdx.x] = 0.0;
    }
}
__global__ void k_cg_direction(CgArgs a) {
    const double beta = a.scal[7];
    for (long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x; f < a.nf; f += (long long)gridDim.x * blockDim.x)
        if (a.inSys[f]) a.p[f] = a.z[f] + beta * a.p[f];
}
// _applySolutionToVelocityField (viscositysolver.cpp:856-891): the field is
// cleared, then the system's faces take the solution.
__global__ void k_visc_write(CgArgs a, float *u, float *v, float *w) {
    const long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= a.nf) return;
    const float val = a.inSys[f] ? (float)a.x[f] : 0.0f;
    if (f < a.s.fx.nu) u[f] = val;
    else if (f < a.s.fx.nu + a.s.fx.nv) v[f - a.s.fx.nu] = val;
    else w[f - a.s.fx.nu - a.s.fx.nv] = val;
}

}  // namespace

void viscosity_buffer_sizes(int I, int J, int K, long long *nf, long long *nn, long long *ncorner,
                            long long vol[7], int *reductionBlocks) {
    const long long nu = (long long)(I + 1) * J * K, nv = (long long)I * (J + 1) * K, nw = (long long)I * J * (K + 1);
    *nf = nu + nv + nw;
    *nn = (long long)(I + 1) * (J + 1) * (K + 1);
    *ncorner = (long long)(I + 2) * (J + 2) * (K + 2);
    const long long g[7][3] = {{I, J, K}, {I + 1, J, K}, {I, J + 1, K}, {I, J, K + 1}, {I, J + 1, K + 1},
                               {I + 1, J, K + 1}, {I + 1, J + 1, K}};
    for (int q = 0; q < 7; q++) vol[q] = g[q][0] * g[q][1] * g[q][2];
    *reductionBlocks = RB;
}

// The viscosity step on the device (buffers from the caller, sized by
// viscosity_buffer_sizes).  Returns FLIP_OK or FLIP_E_CUDA.
int viscosity_apply(const StepConsts &c, const ViscosityBuffers &vb, const float *liquidPhi, const float *solidPhi,
                    float *u, float *v, float *w, double visc, double dt, ViscosityResult *res, cudaStream_t s) {
    const long long nu = (long long)(c.I + 1) * c.J * c.K, nv = (long long)c.I * (c.J + 1) * c.K,
                    nw = (long long)c.I * c.J * (c.K + 1), nf = nu + nv + nw;
    const long long nn = (long long)(c.I + 1) * (c.J + 1) * (c.K + 1);
    { FLIP_COUNT(1); k_visc_states<<<div_up(nf, TPB), TPB, 0, s>>>(c, solidPhi, vb.fluidFace); }
    { FLIP_COUNT(1); k_visc_valid<<<div_up(nn, TPB), TPB, 0, s>>>(c, liquidPhi, vb.valid); }
    { FLIP_COUNT(1); k_visc_dilate<<<div_up(nn, TPB), TPB, 0, s>>>(c, vb.valid, vb.valid2); }
    { FLIP_COUNT(1); k_visc_dilate<<<div_up(nn, TPB), TPB, 0, s>>>(c, vb.valid2, vb.valid); }
    // the seven control-volume grids and their corner offsets (viscositysolver.cpp:240-248)
    const float h = (float)(0.5 * c.dx);
    const VGrid grids[NVOL] = {{c.I, c.J, c.K, h, h, h},         {c.I + 1, c.J, c.K, 0, h, h},
                               {c.I, c.J + 1, c.K, h, 0, h},     {c.I, c.J, c.K + 1, h, h, 0},
                               {c.I, c.J + 1, c.K + 1, h, 0, 0}, {c.I + 1, c.J, c.K + 1, 0, h, 0},
                               {c.I + 1, c.J + 1, c.K, 0, 0, h}};
    VolPtrs vp;
    for (int g = 0; g < NVOL; g++) {
        const VGrid &G = grids[g];
        const long long ncorner = (long long)(G.ni + 1) * (G.nj + 1) * (G.nk + 1), ncell = (long long)G.ni * G.nj * G.nk;
        { FLIP_COUNT(1); k_visc_corners<<<div_up(ncorner, TPB), TPB, 0, s>>>(c, G, vb.valid, liquidPhi, vb.node); }
        { FLIP_COUNT(1); k_visc_volumes<<<div_up(ncell, TPB), TPB, 0, s>>>(c, G, vb.valid, vb.node, vb.vol[g]); }
        vp.v[g] = vb.vol[g];
        vp.ni[g] = G.ni;
        vp.nj[g] = G.nj;
    }
    SysArgs sa;
    sa.fx = FaceIdx{c.I, c.J, c.K, nu, nv};
    sa.vp = vp;
    sa.fluidFace = vb.fluidFace;
    sa.u = u;
    sa.v = v;
    sa.w = w;
    sa.visc = (float)visc;
    const float invdx = (float)(1.0 / c.dx);
    sa.factor = (float)(dt * (double)invdx * (double)invdx);
    { FLIP_COUNT(1); k_visc_rows<<<div_up(nf, TPB), TPB, 0, s>>>(sa, vb.inSys, vb.fac, vb.dr); }
    CgArgs a;
    a.s = sa;
    a.inSys = vb.inSys;
    a.fac = vb.fac;
    a.dr = vb.dr;
    a.nf = nf;
    a.x = vb.x; a.r = vb.r; a.z = vb.z; a.p = vb.p; a.q = vb.q;
    a.part = vb.part;
    a.scal = vb.scal;
    { FLIP_COUNT(1); k_cg_init<<<RB, TPB, 0, s>>>(a); }
    { FLIP_COUNT(1); k_cg_sum<<<1, 1024, 0, s>>>(a, 0); }
    double hs[8];
    cudaError_t e = cudaMemcpyAsync(hs, vb.scal, sizeof(hs), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) { FLIP_SYNC_COUNT(); e = cudaStreamSynchronize(s); }
    if (e != cudaSuccess) return record_error(FLIP_E_CUDA, std::string("viscosity: ") + cudaGetErrorString(e));
    res->rows = (long long)hs[5];
    res->iterations = 0;
    res->residual = 0.0;
    if (res->rows == 0) return FLIP_OK;   // nothing to solve: the field is left as it is (:55-58)
    const double bmax = hs[4], tol = 1e-9 * bmax;
    const int maxIter = 2000, batch = 8;
    double rmax = hs[3];
    int it = 0;
    while (it < maxIter && rmax > tol) {
        for (int q = 0; q < batch; q++) {
            { FLIP_COUNT(1); k_cg_apply<<<RB, TPB, 0, s>>>(a); }
            { FLIP_COUNT(1); k_cg_sum<<<1, 1024, 0, s>>>(a, 1); }
            { FLIP_COUNT(1); k_cg_update<<<RB, TPB, 0, s>>>(a); }
            { FLIP_COUNT(1); k_cg_sum<<<1, 1024, 0, s>>>(a, 2); }
            { FLIP_COUNT(1); k_cg_direction<<<RB, TPB, 0, s>>>(a); }
        }
        it += batch;
        e = cudaMemcpyAsync(hs, vb.scal, sizeof(hs), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) { FLIP_SYNC_COUNT(); e = cudaStreamSynchronize(s); }
        if (e != cudaSuccess) return record_error(FLIP_E_CUDA, std::string("viscosity: ") + cudaGetErrorString(e));
        rmax = hs[3];
    }
    res->iterations = it;
    res->residual = bmax > 0 ? rmax / bmax : 0.0;
    { FLIP_COUNT(1); k_visc_write<<<div_up(nf, TPB), TPB, 0, s>>>(a, u, v, w); }
    e = cudaGetLastError();
    if (e != cudaSuccess) return record_error(FLIP_E_CUDA, std::string("viscosity: ") + cudaGetErrorString(e));
    return FLIP_OK;
}

}  // namespace flip
