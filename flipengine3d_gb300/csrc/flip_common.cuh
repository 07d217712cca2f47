// Shared device helpers for the GB300 FLIP step.
//
// Index and position conventions follow the reference engine so that cell
// keys, block frames and flags come out bit-identical:
//   flat index            i + ni*(j + nj*k)               (array3d.h:425-433)
//   position -> index     floor((double)p * (1.0/dx))     (grid3d.h:56-61)
//   index -> position     (float)((double)(float)i * dx)  (grid3d.h:75-81)
//   cell centre           (float)((double)(float)i*dx + 0.5*dx)  (grid3d.h:99-104)
// The library is compiled with --fmad=false: float expressions that must be
// bit-exact (SDF distances, P2G kernel weights, extrapolation means) are
// evaluated unfused, as the reference's x86-64 build does.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace flip {

struct Dims {
    int ni, nj, nk;
    __host__ __device__ long long size() const { return (long long)ni * nj * nk; }
    __host__ __device__ long long idx(int i, int j, int k) const {
        return (long long)i + (long long)ni * ((long long)j + (long long)nj * k);
    }
    __host__ __device__ bool in(int i, int j, int k) const {
        return i >= 0 && j >= 0 && k >= 0 && i < ni && j < nj && k < nk;
    }
};

// floor((double)p * inv) without FP64 in the common case: the float product
// is within 1.3e-7 relative of the exact one, so away from integer
// boundaries its floor is the exact floor; near them fall back to FP64.
// Kept out of line so the compiler cannot if-convert it into every call.
static __device__ __noinline__ int floor_fp64(float p, double inv) { return (int)floor((double)p * inv); }

__device__ __forceinline__ int exact_floor(float p, double inv, float invf) {
    float q = __fmul_rn(p, invf);
    float fq = floorf(q);
    float frac = __fsub_rn(q, fq);
    float tolf = 1e-3f + 4e-7f * fabsf(q);
    if (frac > tolf && frac < 1.0f - tolf) return (int)fq;
    return floor_fp64(p, inv);
}

__device__ __forceinline__ float idx_to_pos(int i, double dx) { return (float)((double)(float)i * dx); }
__device__ __forceinline__ float cell_centre(int i, double dx) { return (float)((double)(float)i * dx + 0.5 * dx); }

// order-preserving float <-> uint32 encoding for deterministic atomicMin
__device__ __forceinline__ unsigned int f2ord(float f) {
    unsigned int b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned int u) {
    unsigned int b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    return __uint_as_float(b);
}

// Particle key flags (bits above the 28-bit cell index).
constexpr unsigned int KEY_CELL_MASK = 0x0fffffffu;
constexpr unsigned int KEY_SOLID = 0x80000000u;    // removed: inside the solid
constexpr unsigned int KEY_FAST = 0x40000000u;     // over the extreme-speed limit
constexpr unsigned int KEY_NONE = 0xffffffffu;     // no particle

inline unsigned int div_up(long long a, int b) { return (unsigned int)((a + b - 1) / b); }
// Grid coordinates of a flat index i + ni*(j + nj*k).  Grids hold fewer than
// 2^31 entries (flip_create caps them), so 32-bit division suffices; 64-bit
// division has no hardware instruction.
__host__ __device__ __forceinline__ void unflatten(long long t, int ni, int nj, int &i, int &j, int &k) {
    const unsigned u = (unsigned)t, a = (unsigned)ni, b = (unsigned)nj;
    const unsigned q = u / a;
    i = (int)(u - q * a);
    j = (int)(q % b);
    k = (int)(q / b);
}

// The level set of a mesh fluid source over its sub-grid: ni x nj x nk
// nodes, the first at (ox, oy, oz).
struct SourceGridView {
    const float *phi;
    int ni, nj, nk;
    float ox, oy, oz;
    double dx;
};
// MeshLevelSet::trilinearInterpolate (meshlevelset.cpp:261-263, through
// Interpolation::trilinearInterpolate, interpolation.cpp:61-113) at a point
// in the grid's own frame: FP64 weights, corners outside the grid read 0,
// the result rounded to float as the reference returns it.
__device__ __forceinline__ float source_phi(const SourceGridView &g, float px, float py, float pz) {
    const double inv = 1.0 / g.dx;
    const int i = (int)floor((double)px * inv), j = (int)floor((double)py * inv), k = (int)floor((double)pz * inv);
    const float gx = (float)((double)(float)i * g.dx), gy = (float)((double)(float)j * g.dx),
                gz = (float)((double)(float)k * g.dx);
    const double x = (double)__fsub_rn(px, gx) * inv, y = (double)__fsub_rn(py, gy) * inv,
                 z = (double)__fsub_rn(pz, gz) * inv;
    auto at = [&](int a, int b, int c) -> double {
        return (a >= 0 && b >= 0 && c >= 0 && a < g.ni && b < g.nj && c < g.nk)
                   ? (double)g.phi[(long long)a + (long long)g.ni * ((long long)b + (long long)g.nj * c)]
                   : 0.0;
    };
    const double p0 = at(i, j, k), p1 = at(i + 1, j, k), p2 = at(i, j + 1, k), p3 = at(i, j, k + 1),
                 p4 = at(i + 1, j, k + 1), p5 = at(i, j + 1, k + 1), p6 = at(i + 1, j + 1, k),
                 p7 = at(i + 1, j + 1, k + 1);
    return (float)(p0 * (1 - x) * (1 - y) * (1 - z) + p1 * x * (1 - y) * (1 - z) + p2 * (1 - x) * y * (1 - z) +
                   p3 * (1 - x) * (1 - y) * z + p4 * x * (1 - y) * z + p5 * (1 - x) * y * z +
                   p6 * x * y * (1 - z) + p7 * x * y * z);
}
// Inflow sources that constrain the fluid velocity, in registration order
// (fluidsimulation.cpp:3372-3440, 4109-4170).  cellBits: per cell, bit s
// set when the cell is one of source s's cells.
constexpr int MAX_CONSTRAINED_INFLOWS = 8;
struct InflowConstraint {
    int count = 0;
    const uint8_t *cellBits = nullptr;
    SourceGridView g[MAX_CONSTRAINED_INFLOWS];
    float vx[MAX_CONSTRAINED_INFLOWS], vy[MAX_CONSTRAINED_INFLOWS], vz[MAX_CONSTRAINED_INFLOWS];
};

// Count of kernel launches issued by this library (all contexts); each
// launcher adds the number of kernels it enqueues.
long long &launch_counter();
#define FLIP_COUNT(n) (::flip::launch_counter() += (n))
// Host waits on the device (stream or event synchronisations) issued by the
// calling thread, tallied per context like the launches.
long long &host_sync_counter();
#define FLIP_SYNC_COUNT() (++::flip::host_sync_counter())

}  // namespace flip
