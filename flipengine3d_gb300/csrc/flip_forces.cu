// The force-field grid applied to the velocity faces (sm_103a).
//
// FluidSimulation::_applyForceFieldGridForcesThread (fluidsimulation.cpp:
// 3524-3564): every face that no inflow source constrains gains dt times the
// force-field grid at the face position, MACVelocityField::
// evaluateVelocityAtPositionLinearU/V/W (macvelocityfield.cpp:110-160,
// 519-613) on the force-field grid: zero outside its cells, else the FP64
// trilinear interpolation of its faces, with the body force standing in for
// faces outside its range (setOutOfRangeVector, forcefieldgrid.cpp:271).  The
// value is rounded to float, times dt in FP64, and added as a float, as
// MACVelocityField::addU(GridIndex, double) does.
#include "flip_device.cuh"

namespace flip {

namespace {

constexpr int TPB = 256;

// Grid3d::GridIndexToPosition / FaceIndexToPosition (grid3d.h:77-125): FP64
// products rounded to float
__device__ __forceinline__ float ff_node(int i, double dx) { return (float)((double)(float)i * dx); }
__device__ __forceinline__ float ff_centre(int i, double dx) { return (float)(((double)(float)i + 0.5) * dx); }

// MACVelocityField::evaluateVelocityAtPositionLinear{U,V,W} on the grid `f`
__device__ float ff_eval(const ForceFieldView &f, int dir, double x, double y, double z) {
    const double h = f.dx;
    if (!(x >= 0 && y >= 0 && z >= 0 && x < h * f.ni && y < h * f.nj && z < h * f.nk)) return 0.0f;
    if (dir != 0) x -= 0.5 * h;
    if (dir != 1) y -= 0.5 * h;
    if (dir != 2) z -= 0.5 * h;
    const double invdx = 1.0 / h;
    const int i = (int)floor(x * invdx), j = (int)floor(y * invdx), k = (int)floor(z * invdx);
    const double gx = (double)i * h, gy = (double)j * h, gz = (double)k * h;
    const double inv = 1 / h;
    const double ix = (x - gx) * inv, iy = (y - gy) * inv, iz = (z - gz) * inv;
    const float *G = dir == 0 ? f.u : (dir == 1 ? f.v : f.w);
    const int a = f.ni + (dir == 0), b = f.nj + (dir == 1), c = f.nk + (dir == 2);
    const double oor = (double)(dir == 0 ? f.gx : (dir == 1 ? f.gy : f.gz));
    auto val = [&](int ii, int jj, int kk) -> double {
        if (ii < 0 || jj < 0 || kk < 0 || ii >= a || jj >= b || kk >= c) return oor;
        return (double)G[(long long)ii + (long long)a * ((long long)jj + (long long)b * kk)];
    };
    const double p0 = val(i, j, k), p1 = val(i + 1, j, k), p2 = val(i, j + 1, k), p3 = val(i, j, k + 1),
                 p4 = val(i + 1, j, k + 1), p5 = val(i, j + 1, k + 1), p6 = val(i + 1, j + 1, k),
                 p7 = val(i + 1, j + 1, k + 1);
    // Interpolation::trilinearInterpolate(double p[8], x, y, z) (interpolation.cpp:61-70)
    const double r = p0 * (1 - ix) * (1 - iy) * (1 - iz) + p1 * ix * (1 - iy) * (1 - iz) +
                     p2 * (1 - ix) * iy * (1 - iz) + p3 * (1 - ix) * (1 - iy) * iz + p4 * ix * (1 - iy) * iz +
                     p5 * (1 - ix) * iy * iz + p6 * ix * iy * (1 - iz) + p7 * ix * iy * iz;
    return (float)r;
}

__global__ void k_force_field(StepConsts c, float *u, float *v, float *w, ForceFieldView f, double dt,
                              const uint8_t *ex) {
    const long long nu = (long long)(c.I + 1) * c.J * c.K, nv = (long long)c.I * (c.J + 1) * c.K,
                    nw = (long long)c.I * c.J * (c.K + 1);
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nu + nv + nw || (ex && ex[e])) return;
    int dir;
    long long l;
    int a, b;
    if (e < nu) { dir = 0; l = e; a = c.I + 1; b = c.J; }
    else if (e < nu + nv) { dir = 1; l = e - nu; a = c.I; b = c.J + 1; }
    else { dir = 2; l = e - nu - nv; a = c.I; b = c.J; }
    const int i = (int)(l % a), j = (int)((l / a) % b), k = (int)(l / ((long long)a * b));
    const float px = dir == 0 ? ff_node(i, c.dx) : ff_centre(i, c.dx);
    const float py = dir == 1 ? ff_node(j, c.dx) : ff_centre(j, c.dx);
    const float pz = dir == 2 ? ff_node(k, c.dx) : ff_centre(k, c.dx);
    const float force = ff_eval(f, dir, px, py, pz);
    float *G = dir == 0 ? u : (dir == 1 ? v : w);
    G[l] = __fadd_rn(G[l], (float)((double)force * dt));
}

}  // namespace

void launch_force_field(const StepConsts &c, float *u, float *v, float *w, const ForceFieldView &f, double dt,
                        const uint8_t *ex, cudaStream_t s) {
    const long long tot = (long long)(c.I + 1) * c.J * c.K + (long long)c.I * (c.J + 1) * c.K +
                          (long long)c.I * c.J * (c.K + 1);
    FLIP_COUNT(1);
    k_force_field<<<div_up(tot, TPB), TPB, 0, s>>>(c, u, v, w, f, dt, ex);
}

}  // namespace flip
