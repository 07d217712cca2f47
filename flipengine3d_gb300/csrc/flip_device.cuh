// Launch interface of the FLIP step kernels (host side of the CUDA code).
#pragma once
#include <algorithm>
#include <cstdint>
#include <string>
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
    float gxmax, gymax, gzmax;   // largest float coordinate with (double)x < I dx (J dx, K dx)
    double radius;               // liquid SDF / P2G particle radius, 0.5*sqrt(3)*dx
    double cfl;
    int maxPerCell;
    // near-solid coarse grid
    int nsi, nsj, nsk;
    double nearCell, invNearCell;
    float invNearCellf;
    // collision boundary AABB (domain inset, then the solid buffer)
    float bposx, bposy, bposz;
    double bw, bh, bd;
    // position tables (device): node n at (float)((double)(float)n * dx);
    // 10-cell block n at (float)((double)(float)n * 10 dx) and at
    // (float)((double)(float)n * (double)(float)(10 dx)), index n + 1
    const float *nodePos;
    const float *blockPos;
    const float *blockPosF;
};

// -- seeding from fluid meshes (flip_seed.cu); mask: one 8-bit sub-cell
// mask per cell, four cells to a word; owner: 8 I J K words, all ones
void launch_mask_particles(const ParticleSoA &p, int n, const StepConsts &c, unsigned int *mask, cudaStream_t s);
// meshPhi: the mesh's level set, sampled at p minus its first node's position
void launch_seed_candidates(const StepConsts &c, const int *cells, long long ncells, const SourceGridView &meshPhi,
                            const float *solidPhi, double jitter, bool jitterSurface, unsigned long long seed,
                            const unsigned int *mask, float4 *cand, unsigned int *owner, int *keep, cudaStream_t s);
void launch_seed_scatter(const StepConsts &c, long long ncand, const float4 *cand, const int *keep, const int *rank,
                         const ParticleSoA &p, int n0, unsigned int id0, float vx, float vy, float vz,
                         unsigned int *mask, cudaStream_t s);

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
// threads: the CTA size, 256, 512 (default) or 1024
void launch_liquid_sdf(const ParticleSoA &p, const int *cellStart, const StepConsts &c, const uint8_t *solidCC,
                       float *phi, int threads, cudaStream_t s);
void launch_p2g(const ParticleSoA &p, const int *cellStart, const StepConsts &c, float *u, float *v, float *w,
                uint8_t *vu, uint8_t *vv, uint8_t *vw, cudaStream_t s);
void launch_extrapolate(const StepConsts &c, float *u, float *v, float *w, const uint8_t *vu, const uint8_t *vv,
                        const uint8_t *vw, uint8_t *status, int layers, cudaStream_t s);
// The force-field grid on the device (flip_forces.cu): faces of an
// ni x nj x nk grid of cell size dx, and the body force it reads outside them
struct ForceFieldView {
    const float *u, *v, *w;
    int ni, nj, nk;
    double dx;
    float gx, gy, gz;
};
void launch_force_field(const StepConsts &c, float *u, float *v, float *w, const ForceFieldView &f, double dt,
                        const uint8_t *ex, cudaStream_t s);
void launch_save_and_force(const StepConsts &c, float *u, float *v, float *w, float *su, float *sv, float *sw,
                           float fx, float fy, float fz, bool ax, bool ay, bool az, const uint8_t *ex,
                           cudaStream_t s);
void launch_constrain(const StepConsts &c, float *u, float *v, float *w, float *su, float *sv, float *sw,
                      const float *wu, const float *wv, const float *ww, const float *fu, const float *fv,
                      const float *fw, cudaStream_t s);

// -- particle update: PIC/FLIP, RK3, collision, removal tests, new keys
void launch_advect(ParticleSoA p, int n, const StepConsts &c, const float *u, const float *v, const float *w,
                   const float *su, const float *sv, const float *sw, const float *solidPhi,
                   const uint8_t *nearSolid, float picRatio, float flipRatio, double dt, unsigned int *keys,
                   unsigned int *speedHist, double speedStep, const InflowConstraint &ic, cudaStream_t s);

// -- mesh fluid sources (flip_sources.cu)
// Faces (u, v, w, one byte each) that enabled inflow sources constraining the
// fluid velocity keep out of the body force: P2G-valid faces where a
// source's level set, read at the face's position in its own frame, is
// negative (fluidsimulation.cpp:3372-3440).
void launch_inflow_faces(const StepConsts &c, const InflowConstraint &ic, const uint8_t *vu, const uint8_t *vv,
                         const uint8_t *vw, uint8_t *ex, cudaStream_t s);
// Outflow (fluidsimulation.cpp:4608-4650): particles in the source's cells
// (or outside them, inversed) where its level set at p - offset is negative
// (non-negative, inversed) are flagged for removal in keys.
void launch_outflow_mark(const ParticleSoA &p, int n, const StepConsts &c, const uint8_t *cellMask, int inversed,
                         const SourceGridView &g, unsigned int *keys, cudaStream_t s);
void launch_speed_limit(const unsigned int *hist, int n, int bins, double speedStep, double maxPct, int maxAbs,
                        float *maxSpeedSq, cudaStream_t s);
void launch_mark_fast(const ParticleSoA &p, int n, const float *maxSpeedSq, unsigned int *keys, cudaStream_t s);

// -- pressure projection (flip_pcg.cu); dense cell-grid vectors, cells
// outside the system hold zeros
// Sweep layout: the vectors of the MIC(0) sweeps (factor rows, right-hand
// side, result) are stored step-major.  The interior pencils along i are cut
// into tiles of SWEEP_TJ x SWEEP_TK: SWEEP_TJ along the tile's lane axis a
// and SWEEP_TK along its slot axis b, where (a, b) = (j, k), or (k, j) when
// `swap` is set (the orientation is chosen per solve).  Pencil (l, w) of a
// tile holds cell i at forward step tf = i - 1 + SWEEP_SL * l + SWEEP_SW * w:
// a pencil runs SWEEP_SL steps behind its lane neighbour and SWEEP_SW steps
// behind its slot neighbour, so a term crosses lanes SWEEP_SL steps and slots
// SWEEP_SW steps after it is formed.  Entry (tile, tf, w, l) lives at
// ((tile * T + tf) * SWEEP_NP + w * SWEEP_TJ + l),
// T = I - 2 + SWEEP_SL * (SWEEP_TJ - 1) + SWEEP_SW * (SWEEP_TK - 1).  A chunk of
// consecutive steps of a tile is one contiguous block, in either sweep
// direction.  Entries that hold no interior cell stay zero.
#ifndef SWEEP_SL
#define SWEEP_SL 1
#endif
#ifndef SWEEP_SW
#define SWEEP_SW 1
#endif
#ifndef SWEEP_SLOTS
#define SWEEP_SLOTS 8   // pencils of a tile along its slot axis
#endif
constexpr int SWEEP_TJ = 32, SWEEP_TK = SWEEP_SLOTS, SWEEP_NP = SWEEP_TJ * SWEEP_TK;
static_assert(SWEEP_SL >= 1 && SWEEP_SL <= 4 && SWEEP_SW >= 1 && SWEEP_SW <= 4, "sweep skews");
struct SweepLayout {
    int ntj, ntk, T;   // tiles along the lane and warp axes, steps per tile
    int swap;          // 0: lanes along j, warps along k; 1: lanes along k, warps along j
    int EA, EB;        // grid extents along the lane and warp axes
};
inline SweepLayout sweep_layout(int I, int J, int K, int swap = 0) {
    SweepLayout g;
    g.swap = swap;
    g.EA = swap ? K : J;
    g.EB = swap ? J : K;
    g.ntj = (g.EA - 2 + SWEEP_TJ - 1) / SWEEP_TJ;
    g.ntk = (g.EB - 2 + SWEEP_TK - 1) / SWEEP_TK;
    g.T = (I - 2) + SWEEP_SL * (SWEEP_TJ - 1) + SWEEP_SW * (SWEEP_TK - 1);
    return g;
}
// entries of either orientation: the arrays are allocated for the larger
inline long long sweep_layout_size(int I, int J, int K) {
    long long best = 0;
    for (int sw = 0; sw < 2; sw++) {
        SweepLayout g = sweep_layout(I, J, K, sw);
        best = std::max(best, (long long)g.ntj * g.ntk * g.T * SWEEP_NP);
    }
    return best;
}
// entry of interior cell (i, j, k)
__host__ __device__ __forceinline__ long long sweep_index(const SweepLayout &g, int i, int j, int k) {
    const int aa = (g.swap ? k : j) - 1, bb = (g.swap ? j : k) - 1;
    const int l = aa % SWEEP_TJ, w = bb % SWEEP_TK;
    const int tile = aa / SWEEP_TJ + g.ntj * (bb / SWEEP_TK);
    return ((long long)tile * g.T + (i - 1 + SWEEP_SL * l + SWEEP_SW * w)) * SWEEP_NP + w * SWEEP_TJ + l;
}

// Device-side control of the PCG loop: the convergence test runs on the
// device, so the host enqueues iterations in batches and reads this once per
// batch; every kernel of an iteration returns at once when done is set.
struct PcgCtl {
    int done;      // converged
    int iters;     // iterations to convergence
    int claim;     // the recurrence residual passed the test; b - A x must confirm
    int it;        // index of the iteration being run
    unsigned int ticket[4];   // per reduction kernel (spmv, dot_zr, update_xr, true residual): CTAs done
    double resid;  // last residual norm tested
    int batches;     // batches run by the device-side loop
    int maxBatches;  // its limit (maximum iterations / PCG_BATCH)
};
constexpr int PCG_BATCH = 8;   // iterations of a captured batch

struct PressureBuffers {
    uint8_t *fluid;        // interior cell with phi < 0 (a row of the system)
    // the rows as a list, in cell order (built once per solve by a scan):
    // flat index and sweep-layout index of each row, and their number
    int *fluidFlag, *fluidPos, *fluidScan, *nFluid;
    int *fluidIdx, *fluidSk;
    double4_32a *Ad;           // rows {diag, to +x, to +y, to +z}, FP64
    double *b;             // right-hand side (negative divergence)
    double *invdiagD;      // MIC(0) inverse pivots, FP64
    float4 *L;             // {invdiag, Lx, Ly, Lz} for the FP32 sweeps, sweep layout
    float4 *A2;            // per cell {hi, lo}: the rows as exact float pairs (hi + lo = the FP64 value to 48 bits)
    float2 *x, *r, *q;     // solution, residual, A s: exact float pairs {hi, lo} (hi + lo to ~48 bits)
    float *z;              // preconditioned residual, sweep layout
    float *zc;             // the same at the rows in cell order (written by the z.r pass for the SpMV)
    float *s, *s2;         // search direction, double-buffered: an iteration reads one and writes the other
    float *rf;             // r rounded to FP32, the forward sweep's right-hand side, sweep layout
    SweepLayout sl;        // the orientation of the current solve
    long long nsl;         // entries allocated for the sweep layout
    double *partials;      // per-block partial sums (deterministic reduction)
    double *scal;          // [0]=s.q [1]=z.r (new rho) [2]=|b|inf [3]=rho [4]=alpha [5]=beta [6]=tol |b|inf
    unsigned long long *rmaxBits;  // [0] |r|inf of the recurrence, [1] of b - A x, as double bits
    PcgCtl *ctl;
    // PCG_BATCH iterations captured as a CUDA graph, replayed per batch;
    // [1] also records the sweep timing events
    cudaGraphExec_t batchGraph[2][2] = {};   // [timed][orientation]
    long long batchKernels[2][2] = {};
    bool noGraphs = false;   // the stream cannot be captured: launch eagerly
    // untimed solves: the batches inside a device-side loop (a conditional
    // WHILE node), one launch and one host wait per solve
    cudaGraphExec_t loopGraph[2] = {};   // [orientation]
    long long loopKernels[2] = {};       // kernels per pass of the loop body
    bool noLoopGraph = false;            // the loop could not be built: batches from the host
    int *levelRange;       // [0]=min(i+j+k) [1]=max(i+j+k) [2]=system size [3..6]=min/max j, min/max k
    int *factorProgress;   // per factor tile: the last level it finished
    unsigned int *factorTicket;
    float *pressure;       // float copy of x for the velocity update
    int nPartials;
};
struct PressureArgs {
    const float *phi, *wu, *wv, *ww;
    float *u, *v, *w;
    uint8_t *vu, *vv, *vw;
    double dt, tol, accTol;
    int maxIter;
    float *dumpPressure;   // host, optional
    double *dumpRhs;       // host, optional
    struct SweepTiming *sweepTiming;   // optional: event-timed sweep launches
    int sweepOrientation;  // -1: chosen per solve; 0: lanes along j; 1: lanes along k
};
// Device time of the preconditioner sweeps, summed over launches.
struct SweepTiming {
    cudaEvent_t ev[2 * (PCG_BATCH + 1)];   // a pair per sweep pair of a batch, plus the first
    double ms;
    long long launches;     // sweep kernels (forward and backward count one each)
    long long cellSweeps;   // sum over launches of the system rows swept
};
struct PressureMail {      // pinned host scalars
    int levelRange[8];
    double bmax, rho, ptol;
    PcgCtl ctl;
    int sweepErr;
    int maxBatches;
};
struct PressureResult {
    int iterations;
    double residual;
    bool applied;
    int cells;
};

// Bounded device waits: poll rounds of at most ~250 ns each before a wait
// gives up and raises the error flag (about a second).
constexpr unsigned int DEFAULT_SPIN_LIMIT = 1u << 22;

// Pipelined wavefront sweeps (flip_wavefront.cu)
struct SweepState {
    int2 *range;             // per tile [first, last] step holding a system cell
    unsigned long long *xchg;  // tile edge exchange words {epoch, value}
    long long xchgWords;       // words allocated for xchg
    unsigned int *ticket;    // [0] forward tile tickets, [1] the sweep pair's epoch, [2] backward tile tickets
    int *err;                // set when a bounded wait gave up
    unsigned int epoch;      // host count of the epochs issued (wrap guard)
    unsigned int spinLimit = 0;   // poll rounds of the factor's and sweeps' waits (0: DEFAULT_SPIN_LIMIT)
    int stall = 0;           // fault injection: the sweeps' edge waits await an epoch never published
};
int sweep_tiles_max(int I, int J, int K);           // tiles of the larger orientation
long long sweep_exchange_words(int I, int J, int K);   // for the larger orientation
void launch_sweep_ranges(const StepConsts &c, const SweepLayout &g, const uint8_t *fluid, SweepState &sw,
                         cudaStream_t s);
// Before each sweep pair, by one thread of a kernel that runs before it:
// tile tickets from zero for both sweeps and a fresh epoch for each (the
// forward sweep publishes under ticket[1], the backward under ticket[1]+1).
// Kept on the device so that a captured sequence of pairs replays with new
// epochs.
__device__ __forceinline__ void sweep_prep(unsigned int *ticket) {
    ticket[0] = 0u;
    ticket[2] = 0u;
    ticket[1] += 2u;
}
// z = M^-1 r with the MIC(0) factor L: forward then backward sweep
// The launches return at once when *skip is set (a converged solve).
// `prepped`: a kernel ahead of them on the stream already ran sweep_prep.
void launch_sweeps(const StepConsts &c, const SweepLayout &g, const float4 *L, const float *rf, float *z,
                   SweepState &sw, const int *skip, cudaStream_t s, bool prepped = false);
void sweep_epoch_guard(const StepConsts &c, SweepState &sw, long long upcoming, cudaStream_t s);

void mic0_factor(const StepConsts &c, const uint8_t *fluid, const double4_32a *Ad, double *invD, double *W0,
                 double *W1, double *W2, int *progress, unsigned int *ticket, int *err, unsigned int spinLimit,
                 int lo, int hi, cudaStream_t s);
// The reduction grid of the PCG row kernels: one CTA per `cellsPerCta` grid
// cells (a tuning knob, default 4096), at most PCG_MAX_PARTIALS.
constexpr int PCG_MAX_PARTIALS = 152 * 8;
int pressure_partials_for(int I, int J, int K, int cellsPerCta = 4096);
int mic0_factor_tiles(int J, int K);   // tiles of the wavefront factorisation
// PressureSolver::solve (pressuresolver.cpp:44-76) on the device.  Returns
// FLIP_OK (velocities updated, or nothing to solve), FLIP_E_SOLVER_NOCONV
// (left unchanged), FLIP_E_DEVICE_TIMEOUT or FLIP_E_CUDA.
int pressure_project(const StepConsts &c, const PressureArgs &a, PressureBuffers &pb, SweepState &sw,
                     PressureMail *mail, cudaStream_t s, PressureResult *res, std::string *errMsg);

}  // namespace flip

namespace flip {
// -- viscosity (flip_viscosity.cu)
struct ViscosityBuffers {
    uint8_t *fluidFace, *valid, *valid2, *inSys;   // per face; per node (two); per face
    float *node;                                   // corner values of one control-volume grid
    float *vol[7];                                 // control-volume fractions
    float4 *fac, *dr;                              // per face: six factors (two float4); {diag, rhs}
    double *x, *r, *z, *p, *q, *part, *scal;       // CG vectors, partials (3 x blocks), scalars (8)
};
struct ViscosityResult {
    long long rows;
    int iterations;
    double residual;   // |r|inf / |b|inf
};
void viscosity_buffer_sizes(int I, int J, int K, long long *nf, long long *nn, long long *ncorner,
                            long long vol[7], int *reductionBlocks);
int viscosity_apply(const StepConsts &c, const ViscosityBuffers &vb, const float *liquidPhi, const float *solidPhi,
                    float *u, float *v, float *w, double visc, double dt, ViscosityResult *res, cudaStream_t s);

// -- surface reconstruction (flip_mesh.cu)
// The frame of the mesher's one compute chunk: the subdivided grid, its
// blocks of 10^3 nodes, the chunk's nodes and offset, and the particle radii.
struct MeshFrame {
    int I, J, K;
    double dx, invdx, subdx, invsub;
    float invsubf;
    double blockdx, invBlock;      // 10 subdx, occupancy pass
    float invBlockf;
    float blockdxF;                // (float)(10 subdx), the count pass's block size
    double invBlockF;
    float invBlockFf;
    int nbI, nbJ, nbK;             // blocks of the subdivided grid
    int ni, nj, nk;                // chunk nodes
    int cbI, cbJ, cbK;             // chunk blocks
    float offx, offy, offz;        // chunk offset
    float r, sr, maxd;             // radius, search radius, initial distance
    float bbx, bby, bbz;           // the chunk's expanded box
    double bbw, bbh, bbd;
    int solidMode;                 // 0 interpolated, 1 subdivision 2 at offset 0, 2 same grid
    float scalef, invscalef;
};
struct MeshJob {
    StepConsts c;
    ParticleSoA p;
    int n;
    const int *cellStart;
    const float *solidPhi;
    int subdivisions;
    double radius;                 // marker particle radius x marker particle scale
    double smoothValue;
    int smoothIterations;
};
// Device buffers of the mesher, grown on demand; the mesh is verts[cur]
// (nverts xyz floats) and tris (ntris vertex triples).
struct MeshBuffers {
    long long bytes = 0;
    uint8_t *occ = nullptr, *active = nullptr, *cube = nullptr;
    float *field = nullptr;
    int *vstart = nullptr, *tstart = nullptr, *totals = nullptr;
    int2 *tiles = nullptr, *adj = nullptr, *adjStart = nullptr;
    int *adjCursor = nullptr, *adjList = nullptr, *tris = nullptr;
    float *verts[2] = {nullptr, nullptr};
    long long occCap = 0, activeCap = 0, cubeCap = 0, fieldCap = 0, vstartCap = 0, tstartCap = 0, totalsCap = 0,
              tilesCap = 0, adjCap = 0, adjStartCap = 0, adjCursorCap = 0, adjListCap = 0, trisCap = 0;
    long long vertsCap[2] = {0, 0};
    int nverts = 0, ntris = 0, cur = 0;
};
// Mesh the particles of `job` into mb (synchronises the stream twice).
int mesh_surface(const MeshJob &job, MeshBuffers &mb, cudaStream_t s);
void mesh_release(MeshBuffers &mb);
int record_error(int code, const std::string &msg);   // sets flip_last_error()

// Packed xyz positions/velocities (either may be null) of the n particles in
// the reference's order; flags/rank hold idSpace+1 ints, scratch
// scan_scratch_ints(idSpace) ints.
void launch_readback_order(const ParticleSoA &p, int n, int idSpace, int *flags, int *rank, int *scratch,
                           int *total, float *pos, float *vel, cudaStream_t s);
void launch_compact_ids(const ParticleSoA &p, int n, int idSpace, int *flags, int *rank, int *scratch, int *total,
                        cudaStream_t s);
}  // namespace flip
