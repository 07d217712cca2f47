// Launch interface of the FLIP step kernels (host side of the CUDA code).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "flip_common.cuh"

namespace flip {

// Particles, structure of arrays, kept sorted by cell (ascending id inside a
// cell).  `id` is the particle's rank in the reference's load order, which
// the reference preserves through every removal.
struct ParticleSoA {
    float *px, *py, *pz, *vx, *vy, *vz;
    unsigned int *id;
};

struct StepConsts {
    int I, J, K;
    double dx, invdx;
    float invdxf;
    float dxf;
    double radius;        // liquid SDF / P2G particle radius, 0.5*sqrt(3)*dx
    double cfl;
    int maxPerCell;
    // near-solid coarse grid
    int nsi, nsj, nsk;
    double nearCell, invNearCell;
    float invNearCellf;
    // collision boundary AABB (domain inset, then the solid buffer)
    float bposx, bposy, bposz;
    double bw, bh, bd;
};

// -- binning (flip_kernels.cu)
void launch_keys_from_positions(const ParticleSoA &p, int n, const StepConsts &c, unsigned int *keys, cudaStream_t s);
void launch_bin_count(const unsigned int *keys, int n, int *cellCount, cudaStream_t s);
void launch_scan_cells(const int *count, int ncells, int *start, int *blockSums, int *total, cudaStream_t s);
int scan_scratch_ints(int ncells);
void launch_bin_scatter(const unsigned int *keys, int n, const int *cellStart, int *cursor, int *slots, cudaStream_t s);
void launch_cell_sort_select(const int *cellStart, int ncells, int *slots, const unsigned int *ids,
                             const unsigned int *keys, int maxPerCell, int *survivorCount, cudaStream_t s);
void launch_gather_particles(const ParticleSoA &src, ParticleSoA dst, const int *cellStart, const int *slots,
                             const int *newStart, int ncells, unsigned int *maxSpeedSqBits, cudaStream_t s);

// -- grid stages
void launch_liquid_sdf(const ParticleSoA &p, const int *cellStart, const StepConsts &c, const uint8_t *solidCC,
                       float *phi, cudaStream_t s);
void launch_p2g(const ParticleSoA &p, const int *cellStart, const StepConsts &c, float *u, float *v, float *w,
                uint8_t *vu, uint8_t *vv, uint8_t *vw, cudaStream_t s);
void launch_extrapolate(const StepConsts &c, float *u, float *v, float *w, const uint8_t *vu, const uint8_t *vv,
                        const uint8_t *vw, uint8_t *status, int layers, cudaStream_t s);
void launch_save_and_force(const StepConsts &c, float *u, float *v, float *w, float *su, float *sv, float *sw,
                           float fx, float fy, float fz, bool ax, bool ay, bool az, cudaStream_t s);
void launch_constrain(const StepConsts &c, float *u, float *v, float *w, float *su, float *sv, float *sw,
                      const float *wu, const float *wv, const float *ww, cudaStream_t s);

// -- particle update: PIC/FLIP, RK3, collision, removal tests, new keys
void launch_advect(ParticleSoA p, int n, const StepConsts &c, const float *u, const float *v, const float *w,
                   const float *su, const float *sv, const float *sw, const float *solidPhi,
                   const uint8_t *nearSolid, float picRatio, float flipRatio, double dt, unsigned int *keys,
                   unsigned int *speedHist, double speedStep, cudaStream_t s);
void launch_speed_limit(const unsigned int *hist, int n, int bins, double speedStep, double maxPct, int maxAbs,
                        float *maxSpeedSq, cudaStream_t s);
void launch_mark_fast(const ParticleSoA &p, int n, const float *maxSpeedSq, unsigned int *keys, cudaStream_t s);

// -- pressure (flip_pressure.cu)
// Dense cell-grid vectors; cells outside the pressure system hold zeros.
struct PressureBuffers {
    uint8_t *fluid;        // interior cell with phi < 0 (a row of the system)
    float4 *A;             // {diag, to +x, to +y, to +z} coefficients, FP32
    double *Adiag;         // diagonal, FP64
    double *b;             // right-hand side (negative divergence), FP64
    double *invdiagD;      // MIC(0) inverse pivots, FP64 (factorisation)
    float4 *L;             // {invdiag, Lx, Ly, Lz} for the FP32 sweeps
    double *x;             // solution, FP64
    float *r, *z, *s, *q;  // CG vectors, FP32
    double *partials;      // per-block partial sums (deterministic reduction)
    double *scal;          // [0]=s.q  [1]=z.r (new rho)  [2]=|b|inf  [3]=rho
    unsigned int *rmaxBits;// |r|inf as float bits
    int *levelRange;       // [0]=min(i+j+k) [1]=max(i+j+k) over system cells, [2]=count
    float *pressure;       // float copy of x for the velocity update
    int nPartials;
};
int pressure_partials(const StepConsts &c);
void launch_pressure_build(const StepConsts &c, const float *phi, const float *wu, const float *wv,
                           const float *ww, const float *u, const float *v, const float *w, double dt,
                           PressureBuffers &pb, cudaStream_t s);
void launch_mic0_factor(const StepConsts &c, const float *phi, const float *wu, const float *wv, const float *ww,
                        double dt, PressureBuffers &pb, int levelLo, int levelHi, cudaStream_t s);
void launch_precondition(const StepConsts &c, PressureBuffers &pb, const float *rin, float *zout, int levelLo,
                         int levelHi, cudaStream_t s);
void launch_spmv_dot(const StepConsts &c, PressureBuffers &pb, cudaStream_t s);       // q = A s, scal[0] = s.q
void launch_dot_zr(const StepConsts &c, PressureBuffers &pb, cudaStream_t s);         // scal[1] = z.r
void launch_update_xr(const StepConsts &c, PressureBuffers &pb, cudaStream_t s);      // alpha = scal[3]/scal[0]
void launch_init_residual(const StepConsts &c, PressureBuffers &pb, cudaStream_t s);  // r = b, |r|inf
void launch_set_rho(PressureBuffers &pb, cudaStream_t s);                             // scal[3] = scal[1]
void launch_copy_zs(const StepConsts &c, PressureBuffers &pb, cudaStream_t s);        // s = z
// out = b - A x with FP64 rows (x FP64), |out|inf into *rmaxOut
void launch_true_residual(const StepConsts &c, const float *phi, const float *wu, const float *wv,
                          const float *ww, double dt, PressureBuffers &pb, float *out, unsigned int *rmaxOut,
                          cudaStream_t s);
void launch_copy_qr(const StepConsts &c, PressureBuffers &pb, cudaStream_t s);        // r = q
void launch_update_s(const StepConsts &c, PressureBuffers &pb, cudaStream_t s);       // beta = scal[1]/scal[3]
void launch_pressure_to_float(const StepConsts &c, PressureBuffers &pb, cudaStream_t s);
void launch_apply_pressure(const StepConsts &c, const float *phi, const float *wu, const float *wv,
                           const float *ww, const PressureBuffers &pb, double dt, float *u, float *v, float *w,
                           uint8_t *vu, uint8_t *vv, uint8_t *vw, cudaStream_t s);

}  // namespace flip
