// Host side of the GB300 FLIP step: the context behind the C ABI in
// include/flip3d.h, device memory, the frame/substep loop of
// FluidSimulation::update (src/engine/fluidsimulation.cpp:5755-5845) and the
// stage sequence of _stepFluid (:5471-5508), each stage a CUDA kernel.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/flip3d.h"
#include "flip_device.cuh"
#include "force_fields.h"
#include "solid_setup.h"

namespace flip {
// Kernel launches issued by the calling thread; each context adds the
// launches of its own calls (LaunchTally), so contexts driven from
// different threads keep separate counts.
long long &launch_counter() {
    static thread_local long long n = 0;
    return n;
}
long long &host_sync_counter() {
    static thread_local long long n = 0;
    return n;
}
}  // namespace flip

using namespace flip;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

#define CK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) return fail(FLIP_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <class T>
int dalloc(T **p, size_t count) {
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)p, count * sizeof(T));
    if (e != cudaSuccess) return fail(FLIP_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return FLIP_OK;
}

}  // namespace

struct flip_ctx {
    int I, J, K;
    double dx;
    int device = 0;
    cudaStream_t stream = nullptr;
    bool ownStream = false;

    // parameters (reference defaults, fluidsimulation.h:1519-1700)
    double picRatio = 0.05;
    std::vector<float> bodyForces;   // xyz triples
    double cfl = 5.0;
    double tol = 1e-9, accTol = 1.0;
    int maxIter = 1000;
    int minFrameSteps = 1, maxFrameSteps = 6;
    int maxPerCell = 250;
    double maxRemovePct = 0.0005;
    int maxRemoveAbs = 35;

    // state
    bool initialized = false;
    std::vector<float> queuePos, queueVel;
    const float *queueDevPos = nullptr, *queueDevVel = nullptr;
    int queueDevN = 0;
    int n = 0, capacity = 0;
    int frame = 0, stepNumber = 0;
    double frameDt = 0, frameRemaining = 0;
    bool outputInitialized = false;
    bool solidBuilt = false;
    flip_frame_stats stats{};
    double maxSpeed = 0.0;

    DomainBox box;
    std::vector<MeshObstacle> obstacles;   // static mesh obstacles (addMeshObstacle)
    // fluid meshes queued by addMeshFluid, seeded at the end of the next substep
    struct FluidMesh {
        std::vector<float> verts;
        std::vector<int> tris;
        float vx, vy, vz;
    };
    std::vector<FluidMesh> fluidQueue;
    // mesh fluid sources (addMeshFluidSource), static meshes
    struct FluidSource {
        int id = 0;
        std::vector<float> verts;
        std::vector<int> tris;
        flip_fluid_source_params prm{};
        SourceGrid grid;           // host set-up, once
        bool built = false;
        float *dphi = nullptr;     // the level set on the device
        int *dcells = nullptr;     // the cells, ascending
        uint8_t *dmask = nullptr;  // one byte per grid cell: 1 for the source's cells
    };
    std::vector<FluidSource> sources;
    int nextSourceId = 0;
    uint8_t *inflowFaces = nullptr;      // faces kept out of the body force (u, v, w)
    uint8_t *inflowCellBits = nullptr;   // per cell: bit q for constraining inflow q
    std::vector<int> cellBitsIds;        // the sources inflowCellBits was built for, in order
    double jitterFactor = 0.0;      // _markerParticleJitterFactor
    bool jitterSurface = false;     // _isJitterSurfaceMarkerParticlesEnabled
    unsigned long long seedCalls = 0;
    unsigned int idNext = 0;        // ids handed out so far (loaded, then seeded)
    float *fu = nullptr, *fv = nullptr, *fw = nullptr;   // face friction, when an obstacle has some
    StepConsts c{};
    // surface reconstruction (fluidsimulation.h:1586-1611: on, subdivision
    // 1, smoothing 0.5 x 2, marker particle scale 3)
    bool meshEnabled = true;
    int meshSubdivisions = 1;
    double meshSmoothValue = 0.5;
    int meshSmoothIterations = 2;
    double markerParticleScale = 3.0;
    MeshBuffers mesh;
    // viscosity (setViscosity, fluidsimulation.cpp:1654-1670): off until set
    bool viscosityEnabled = false;
    double viscosity = 0.0;
    ViscosityBuffers vb{};
    bool vbReady = false;
    ViscosityResult viscResult{};
    // force fields (enableForceFields, fluidsimulation.cpp:1605-1647): point
    // fields; the grid is rebuilt on the host at the first substep of a frame
    // after a change (ffDirty, or the body force moved) and uploaded
    struct ForceFieldEntry {
        int id;
        flip::PointForceField f;
    };
    bool ffEnabled = false;
    int ffReduction = 1;
    std::vector<ForceFieldEntry> forceFields;
    int nextForceFieldId = 0;
    bool ffDirty = true;
    bool ffGravitySet = false;
    float ffGravity[3] = {0.f, 0.f, 0.f};
    flip::ForceFieldGridHost ffHost;
    float *ffU = nullptr, *ffV = nullptr, *ffW = nullptr;
    // tuning knobs (flip_set_tuning): liquid-SDF CTA size, grid cells per
    // CTA of the PCG row kernels; neither changes the results' meaning
    int sdfThreads = 512;
    int pcgCellsPerCta = 4096;

    // device buffers
    ParticleSoA pa{}, pb{};
    unsigned int *keys = nullptr;
    int idSpace = 0;   // ids are ranks in the load order, below idSpace
    int *idFlags = nullptr, *idRank = nullptr, *idScratch = nullptr, *idTotal = nullptr;
    int *cellCount = nullptr, *cellStart = nullptr, *cursor = nullptr, *slots = nullptr;
    int *survivors = nullptr, *newStart = nullptr, *scanScratch = nullptr, *scanTotal = nullptr;
    float *phi = nullptr, *solidPhi = nullptr, *wu = nullptr, *wv = nullptr, *ww = nullptr;
    uint8_t *solidCC = nullptr, *nearSolid = nullptr;
    float *u = nullptr, *v = nullptr, *w = nullptr, *su = nullptr, *sv = nullptr, *sw = nullptr;
    uint8_t *vu = nullptr, *vv = nullptr, *vw = nullptr, *status = nullptr;
    PressureBuffers pr{};
    SweepState sweep{};
    unsigned int *speedHist = nullptr, *maxVelSqBits = nullptr;
    float *maxSpeedSq = nullptr;
    // pinned host mailbox for per-substep scalars
    struct Mail {
        int levelRange[8];
        double bmax;
        double rho;
        unsigned int rmaxBits;
        int total;
        unsigned int velSqBits;
        int sweepErr;
    } *mail = nullptr;
    PressureMail *pmail = nullptr;
    std::vector<void *> allocations;
    std::vector<size_t> allocationBytes;

    long long launches = 0;      // kernel launches of this context's calls
    long long hostSyncs = 0;     // host waits on the device in this context's calls
    long long deviceBytes = 0;   // device memory allocated for this context

    // stage timing
    bool timing = false;
    int sweepOrientation = -1;
    bool endMarkPending = false;
    cudaEvent_t ev[FLIP_NUM_STAGES + 1] = {};
    double stageMs[FLIP_NUM_STAGES] = {};
    long long timedSubsteps = 0;
    SweepTiming sweepTiming{};
    void mark(int stage) {
        if (timing) cudaEventRecord(ev[stage], stream);
    }

    long long nu() const { return (long long)(I + 1) * J * K; }
    long long nv() const { return (long long)I * (J + 1) * K; }
    long long nw() const { return (long long)I * J * (K + 1); }
    long long nc() const { return (long long)I * J * K; }

    template <class T>
    int alloc(T **p, size_t count) {
        int rc = dalloc(p, count);
        if (rc == FLIP_OK) {
            allocations.push_back((void *)*p);
            allocationBytes.push_back(std::max<size_t>(count, 1) * sizeof(T));
            deviceBytes += (long long)allocationBytes.back();
        }
        return rc;
    }
    void release(void *p) {
        for (size_t q = 0; q < allocations.size(); q++)
            if (allocations[q] == p) {
                cudaFree(p);
                deviceBytes -= (long long)allocationBytes[q];
                allocations.erase(allocations.begin() + q);
                allocationBytes.erase(allocationBytes.begin() + q);
                return;
            }
    }
};

// adds the launches and host synchronisations made during one call to the
// context's counts
struct LaunchTally {
    flip_ctx *x;
    long long start, syncStart;
    explicit LaunchTally(flip_ctx *c)
        : x(c), start(flip::launch_counter()), syncStart(flip::host_sync_counter()) {}
    ~LaunchTally() {
        if (x) {
            x->launches += flip::launch_counter() - start;
            x->hostSyncs += flip::host_sync_counter() - syncStart;
        }
    }
};

namespace {

int sync(flip_ctx *x) {
    FLIP_SYNC_COUNT();
    cudaError_t e = cudaStreamSynchronize(x->stream);
    if (e != cudaSuccess) return fail(FLIP_E_CUDA, std::string("stream: ") + cudaGetErrorString(e));
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(FLIP_E_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    return FLIP_OK;
}

float3 body_force(const flip_ctx *x) {
    // _getConstantBodyForce (fluidsimulation.cpp:3363-3370): float sum
    float bx = 0.f, by = 0.f, bz = 0.f;
    for (size_t q = 0; q + 2 < x->bodyForces.size(); q += 3) {
        bx += x->bodyForces[q];
        by += x->bodyForces[q + 1];
        bz += x->bodyForces[q + 2];
    }
    return make_float3(bx, by, bz);
}

int alloc_grids(flip_ctx *x) {
    int rc;
    long long nc = x->nc();
    if ((rc = x->alloc(&x->cellCount, nc + 1))) return rc;
    if ((rc = x->alloc(&x->cellStart, nc + 1))) return rc;
    if ((rc = x->alloc(&x->cursor, nc + 1))) return rc;
    if ((rc = x->alloc(&x->survivors, nc + 1))) return rc;
    if ((rc = x->alloc(&x->newStart, nc + 1))) return rc;
    if ((rc = x->alloc(&x->scanScratch, scan_scratch_ints((int)nc) + 4))) return rc;
    if ((rc = x->alloc(&x->scanTotal, 4))) return rc;
    if ((rc = x->alloc(&x->phi, nc))) return rc;
    if ((rc = x->alloc(&x->solidPhi, (size_t)(x->I + 1) * (x->J + 1) * (x->K + 1)))) return rc;
    if ((rc = x->alloc(&x->solidCC, nc))) return rc;
    if ((rc = x->alloc(&x->wu, x->nu())) || (rc = x->alloc(&x->wv, x->nv())) || (rc = x->alloc(&x->ww, x->nw())))
        return rc;
    if ((rc = x->alloc(&x->u, x->nu())) || (rc = x->alloc(&x->v, x->nv())) || (rc = x->alloc(&x->w, x->nw())))
        return rc;
    if ((rc = x->alloc(&x->su, x->nu())) || (rc = x->alloc(&x->sv, x->nv())) || (rc = x->alloc(&x->sw, x->nw())))
        return rc;
    if ((rc = x->alloc(&x->vu, x->nu())) || (rc = x->alloc(&x->vv, x->nv())) || (rc = x->alloc(&x->vw, x->nw())))
        return rc;
    if ((rc = x->alloc(&x->status, x->nu() + x->nv() + x->nw()))) return rc;
    PressureBuffers &p = x->pr;
    const long long nsl = sweep_layout_size(x->I, x->J, x->K);
    p.sl = sweep_layout(x->I, x->J, x->K, 0);
    p.nsl = nsl;
    if ((rc = x->alloc(&p.fluid, nc)) || (rc = x->alloc(&p.Ad, nc)) || (rc = x->alloc(&p.L, nsl)) ||
        (rc = x->alloc(&p.b, nc)) || (rc = x->alloc(&p.invdiagD, nc)) || (rc = x->alloc(&p.x, nc)) ||
        (rc = x->alloc(&p.r, nc)) || (rc = x->alloc(&p.q, nc)) || (rc = x->alloc(&p.z, nsl)) ||
        (rc = x->alloc(&p.zc, nc)) ||
        (rc = x->alloc(&p.A2, 2 * nc)) ||
        (rc = x->alloc(&p.s, nc)) || (rc = x->alloc(&p.s2, nc)) || (rc = x->alloc(&p.rf, nsl)) ||
        (rc = x->alloc(&p.pressure, nc)))
        return rc;
    if ((rc = x->alloc(&p.fluidFlag, nc + 1)) || (rc = x->alloc(&p.fluidPos, nc + 1)) ||
        (rc = x->alloc(&p.fluidScan, scan_scratch_ints((int)nc) + 4)) || (rc = x->alloc(&p.nFluid, 4)) ||
        (rc = x->alloc(&p.fluidIdx, nc)) || (rc = x->alloc(&p.fluidSk, nc)))
        return rc;
    // entries of the sweep layout that hold no interior cell stay zero
    CK(cudaMemsetAsync(p.L, 0, nsl * sizeof(float4), x->stream));
    CK(cudaMemsetAsync(p.rf, 0, nsl * sizeof(float), x->stream));
    CK(cudaMemsetAsync(p.z, 0, nsl * sizeof(float), x->stream));
    CK(cudaMemsetAsync(p.zc, 0, nc * sizeof(float), x->stream));
    p.nPartials = pressure_partials_for(x->I, x->J, x->K, x->pcgCellsPerCta);
    if ((rc = x->alloc(&p.partials, PCG_MAX_PARTIALS + 32)) || (rc = x->alloc(&p.scal, 8)) ||
        (rc = x->alloc(&p.rmaxBits, 2)) || (rc = x->alloc(&p.levelRange, 8)) || (rc = x->alloc(&p.ctl, 1)) ||
        (rc = x->alloc(&p.factorProgress, mic0_factor_tiles(x->J, x->K))) || (rc = x->alloc(&p.factorTicket, 1)))
        return rc;
    {
        int nt = sweep_tiles_max(x->I, x->J, x->K);
        long long nw = sweep_exchange_words(x->I, x->J, x->K);
        x->sweep.xchgWords = nw;
        if ((rc = x->alloc(&x->sweep.range, nt)) || (rc = x->alloc(&x->sweep.xchg, nw)) ||
            (rc = x->alloc(&x->sweep.ticket, 4)) || (rc = x->alloc(&x->sweep.err, 4)))
            return rc;
        CK(cudaMemsetAsync(x->sweep.xchg, 0, nw * sizeof(unsigned long long), x->stream));
        CK(cudaMemsetAsync(x->sweep.err, 0, 4 * sizeof(int), x->stream));
        CK(cudaMemsetAsync(x->sweep.ticket, 0, 4 * sizeof(unsigned int), x->stream));
    }
    {
        // position tables (see StepConsts)
        int nmax = std::max(x->I, std::max(x->J, x->K)) + 16;
        int nb = nmax / 10 + 4;
        std::vector<float> node(nmax), blk(nb), blkf(nb);
        for (int q = 0; q < nmax; q++) node[q] = (float)((double)(float)q * x->dx);
        float bdx = (float)(10 * x->dx);
        for (int q = 0; q < nb; q++) {
            blk[q] = (float)((double)(float)(q - 1) * (10.0 * x->dx));
            blkf[q] = (float)((double)(float)(q - 1) * (double)bdx);
        }
        float *dn, *db, *dbf;
        if ((rc = x->alloc(&dn, nmax)) || (rc = x->alloc(&db, nb)) || (rc = x->alloc(&dbf, nb))) return rc;
        CK(cudaMemcpy(dn, node.data(), nmax * 4, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(db, blk.data(), nb * 4, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(dbf, blkf.data(), nb * 4, cudaMemcpyHostToDevice));
        x->c.nodePos = dn;
        x->c.blockPos = db;
        x->c.blockPosF = dbf;
    }
    if ((rc = x->alloc(&x->speedHist, 8)) || (rc = x->alloc(&x->maxVelSqBits, 4)) || (rc = x->alloc(&x->maxSpeedSq, 4)))
        return rc;
    CK(cudaMemsetAsync(x->phi, 0, nc * sizeof(float), x->stream));
    CK(cudaMemsetAsync(x->u, 0, x->nu() * 4, x->stream));
    CK(cudaMemsetAsync(x->v, 0, x->nv() * 4, x->stream));
    CK(cudaMemsetAsync(x->w, 0, x->nw() * 4, x->stream));
    return FLIP_OK;
}

int alloc_particles(flip_ctx *x, int cap) {
    int rc;
    x->capacity = cap;
    x->idSpace = cap;
    ParticleSoA *bufs[2] = {&x->pa, &x->pb};
    for (ParticleSoA *b : bufs) {   // one block per buffer: 6 float planes then the ids
        float *base;
        if ((rc = x->alloc(&base, 7 * (size_t)cap))) return rc;
        b->px = base; b->py = base + cap; b->pz = base + 2 * (size_t)cap;
        b->vx = base + 3 * (size_t)cap; b->vy = base + 4 * (size_t)cap; b->vz = base + 5 * (size_t)cap;
        b->id = (unsigned int *)(base + 6 * (size_t)cap);
    }
    if ((rc = x->alloc(&x->keys, cap)) || (rc = x->alloc(&x->slots, cap))) return rc;
    if ((rc = x->alloc(&x->idFlags, cap + 1)) || (rc = x->alloc(&x->idRank, cap + 1)) ||
        (rc = x->alloc(&x->idScratch, scan_scratch_ints(cap) + 4)) || (rc = x->alloc(&x->idTotal, 4)))
        return rc;
    return FLIP_OK;
}

int rebin(flip_ctx *x);

// Larger particle storage, keeping the n particles of `pa` (seeding adds
// particles after initialize; the stream is idle when this is called).
int grow_particles(flip_ctx *x, int cap) {
    if (cap <= x->capacity) return FLIP_OK;
    // a quarter more than asked for, so that steady emission grows the
    // storage rarely
    cap = (int)std::min<long long>(std::max<long long>(cap, (long long)x->capacity * 5 / 4), 0x7ffffff0LL);
    ParticleSoA keep = x->pa;
    const int oldCap = x->capacity;
    void *old[] = {x->pa.px, x->pb.px, x->keys, x->slots, x->idFlags, x->idRank, x->idScratch, x->idTotal};
    int rc = alloc_particles(x, cap);
    if (rc) return rc;
    cudaStream_t s = x->stream;
    if (x->n > 0) {   // the six float planes and the ids of pa
        for (int q = 0; q < 7; q++)
            CK(cudaMemcpyAsync(x->pa.px + (size_t)q * cap, keep.px + (size_t)q * oldCap, (size_t)x->n * 4,
                               cudaMemcpyDeviceToDevice, s));
    }
    if ((rc = sync(x))) return rc;
    for (void *p : old) x->release(p);
    return FLIP_OK;
}

// The device copies of each source's set-up (cells, level set), made once.
int prepare_sources(flip_ctx *x) {
    for (auto &src : x->sources) {
        if (src.built) continue;
        fluid_source_setup(x->I, x->J, x->K, x->dx, src.verts, src.tris, src.grid);
        int rc;
        if ((rc = x->alloc(&src.dphi, src.grid.phi.size())) || (rc = x->alloc(&src.dcells, src.grid.cells.size())) ||
            (rc = x->alloc(&src.dmask, (size_t)x->nc())))
            return rc;
        std::vector<uint8_t> mask((size_t)x->nc(), 0);
        for (int q : src.grid.cells) mask[q] = 1;
        CK(cudaMemcpy(src.dphi, src.grid.phi.data(), src.grid.phi.size() * 4, cudaMemcpyHostToDevice));
        if (!src.grid.cells.empty())
            CK(cudaMemcpy(src.dcells, src.grid.cells.data(), src.grid.cells.size() * 4, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(src.dmask, mask.data(), mask.size(), cudaMemcpyHostToDevice));
        src.built = true;
    }
    return FLIP_OK;
}

SourceGridView source_view(const flip_ctx *x, const flip_ctx::FluidSource &src) {
    SourceGridView g;
    g.phi = src.dphi;
    g.ni = src.grid.nodes[0];
    g.nj = src.grid.nodes[1];
    g.nk = src.grid.nodes[2];
    g.ox = src.grid.offset[0];
    g.oy = src.grid.offset[1];
    g.oz = src.grid.offset[2];
    g.dx = x->dx;
    return g;
}

// The enabled inflow sources that constrain the fluid velocity, in
// registration order, with the per-cell bits of their cells.
int inflow_constraint(flip_ctx *x, InflowConstraint *ic) {
    *ic = InflowConstraint{};
    std::vector<int> ids;
    for (auto &src : x->sources)
        if (src.prm.enabled && src.prm.inflow && src.prm.constrained_velocity) ids.push_back(src.id);
    if (ids.empty()) return FLIP_OK;
    int rc;
    if ((rc = prepare_sources(x))) return rc;
    if (!x->inflowFaces && (rc = x->alloc(&x->inflowFaces, (size_t)(x->nu() + x->nv() + x->nw())))) return rc;
    if (!x->inflowCellBits && (rc = x->alloc(&x->inflowCellBits, (size_t)x->nc()))) return rc;
    if (ids != x->cellBitsIds) {
        std::vector<uint8_t> bits((size_t)x->nc(), 0);
        int q = 0;
        for (auto &src : x->sources)
            if (src.prm.enabled && src.prm.inflow && src.prm.constrained_velocity) {
                for (int cell : src.grid.cells) bits[cell] |= (uint8_t)(1u << q);
                q++;
            }
        CK(cudaMemcpyAsync(x->inflowCellBits, bits.data(), bits.size(), cudaMemcpyHostToDevice, x->stream));
        FLIP_SYNC_COUNT();
        CK(cudaStreamSynchronize(x->stream));
        x->cellBitsIds = ids;
    }
    ic->cellBits = x->inflowCellBits;
    for (auto &src : x->sources)
        if (src.prm.enabled && src.prm.inflow && src.prm.constrained_velocity) {
            const int q = ic->count++;
            ic->g[q] = source_view(x, src);
            ic->vx[q] = (float)src.prm.velocity[0];
            ic->vy[q] = (float)src.prm.velocity[1];
            ic->vz[q] = (float)src.prm.velocity[2];
        }
    return FLIP_OK;
}

// _updateFluidObjects (fluidsimulation.cpp:4794-4806) after a substep: the
// queued fluid meshes (_updateAddedFluidMeshObjectQueue, :4724-4759), then
// the inflow sources' emission (_updateInflowMeshFluidSources, :4676-4698,
// 4564-4606) and the outflow sources' removal (_updateOutflowMeshFluidSources,
// :4700-4717, 4608-4674).  Cells and level sets come from the host set-up;
// particles are seeded on the device (flip_seed.cu) into one sub-cell mask
// shared by every emission, outflow removal flags the particles in their
// keys, and one binning orders everything.
int update_fluid_objects(flip_ctx *x) {
    int rc;
    std::vector<const flip_ctx::FluidSource *> emit;
    bool outflow = false;
    for (auto &src : x->sources) {
        if (!src.prm.enabled) continue;
        if (!src.prm.inflow) {
            outflow = outflow || src.prm.fluid_outflow;
            continue;
        }
        int e = src.prm.substep_emissions;
        if (e == 0) {   // only at a frame's first substep
            if (x->stepNumber != 0) continue;
            e = 1;
        }
        for (int q = 0; q < e; q++) emit.push_back(&src);
    }
    if (x->fluidQueue.empty() && emit.empty() && !outflow) return FLIP_OK;
    if ((rc = prepare_sources(x))) return rc;
    cudaStream_t s = x->stream;
    const long long nc = x->nc();
    std::vector<std::vector<int>> cells(x->fluidQueue.size());
    std::vector<std::vector<float>> phi(x->fluidQueue.size());
    long long ncand = 0, maxCand = 0, queueCand = 0;
    for (size_t m = 0; m < x->fluidQueue.size(); m++) {
        mesh_fluid_cells(x->I, x->J, x->K, x->dx, x->fluidQueue[m].verts, x->fluidQueue[m].tris, cells[m], phi[m]);
        ncand += 8 * (long long)cells[m].size();
        queueCand = std::max(queueCand, 8 * (long long)cells[m].size());
    }
    maxCand = queueCand;
    for (const auto *src : emit) {
        ncand += 8 * (long long)src->grid.cells.size();
        maxCand = std::max(maxCand, 8 * (long long)src->grid.cells.size());
    }
    if ((long long)x->n + ncand >= 0x7fffffffLL || (long long)x->idNext + ncand >= 0x7fffffffLL)
        return fail(FLIP_E_OUT_OF_RANGE, "too many particles");
    if (ncand > 0) {
        // ids are ranks below the id space, which is the storage's capacity:
        // once emission and removal have spread them out, renumber them
        if ((long long)x->idNext + ncand > x->capacity && x->idNext > (unsigned int)x->n) {
            launch_compact_ids(x->pa, x->n, x->idSpace, x->idFlags, x->idRank, x->idScratch, x->idTotal, s);
            x->idNext = (unsigned int)x->n;
        }
        if ((rc = grow_particles(x, std::max(x->capacity, (int)(x->idNext + ncand))))) return rc;
    }
    // scratch of this call only
    struct Scratch {
        std::vector<void *> p;
        ~Scratch() { for (void *q : p) cudaFree(q); }
    } sc;
    auto get = [&](auto **ptr, long long count) {
        if (dalloc(ptr, (size_t)std::max(count, 1LL))) return false;
        sc.p.push_back((void *)*ptr);
        return true;
    };
    if (ncand > 0) {
        unsigned int *mask, *owner;
        float4 *cand;
        int *dcells, *keep, *rank, *scratch, *total;
        float *dphi = nullptr;
        const long long nphi = (long long)(x->I + 1) * (x->J + 1) * (x->K + 1);
        if (!get(&mask, (nc + 3) / 4) || !get(&owner, 8 * nc) || !get(&cand, maxCand) ||
            !get(&dcells, queueCand / 8) || !get(&keep, maxCand) || !get(&rank, maxCand + 1) ||
            !get(&scratch, scan_scratch_ints((int)maxCand) + 4) || !get(&total, 4) ||
            (!x->fluidQueue.empty() && !get(&dphi, nphi)))
            return fail(FLIP_E_NOMEM, "cudaMalloc failed (seeding)");
        CK(cudaMemsetAsync(mask, 0, (size_t)((nc + 3) / 4) * 4, s));
        launch_mask_particles(x->pa, x->n, x->c, mask, s);
        const double jitter = 0.25 * (x->jitterFactor - 1e-3) * x->dx;   // _getMarkerParticleJitter
        const size_t jobs = x->fluidQueue.size() + emit.size();
        for (size_t m = 0; m < jobs; m++) {
            const bool queued = m < x->fluidQueue.size();
            const flip_ctx::FluidSource *src = queued ? nullptr : emit[m - x->fluidQueue.size()];
            const long long ncells = queued ? (long long)cells[m].size() : (long long)src->grid.cells.size();
            const long long nm = 8 * ncells;
            if (nm == 0) continue;
            SourceGridView g;
            const int *dc;
            float vx, vy, vz;
            if (queued) {
                const auto &fm = x->fluidQueue[m];
                CK(cudaMemcpyAsync(dcells, cells[m].data(), cells[m].size() * 4, cudaMemcpyHostToDevice, s));
                CK(cudaMemcpyAsync(dphi, phi[m].data(), (size_t)nphi * 4, cudaMemcpyHostToDevice, s));
                g = SourceGridView{dphi, x->I + 1, x->J + 1, x->K + 1, 0.0f, 0.0f, 0.0f, x->dx};
                dc = dcells;
                vx = fm.vx; vy = fm.vy; vz = fm.vz;
            } else {
                g = source_view(x, *src);
                dc = src->dcells;
                vx = (float)src->prm.velocity[0]; vy = (float)src->prm.velocity[1]; vz = (float)src->prm.velocity[2];
            }
            CK(cudaMemsetAsync(owner, 0xff, (size_t)(8 * nc) * 4, s));
            const unsigned long long seed = 0x5eed5eed5eed5eedull ^ (++x->seedCalls * 0x2545f4914f6cdd1dull);
            launch_seed_candidates(x->c, dc, ncells, g, x->solidPhi, jitter, x->jitterSurface, seed, mask, cand,
                                   owner, keep, s);
            launch_scan_cells(keep, (int)nm, rank, scratch, total, s);
            CK(cudaMemcpyAsync(&x->mail->total, total, sizeof(int), cudaMemcpyDeviceToHost, s));
            if ((rc = sync(x))) return rc;   // the cells and level set buffers are reused for the next mesh
            const int added = x->mail->total;
            launch_seed_scatter(x->c, nm, cand, keep, rank, x->pa, x->n, x->idNext, vx, vy, vz, mask, s);
            x->n += added;
            x->idNext += (unsigned int)added;
        }
    }
    x->fluidQueue.clear();
    // bin everything (every particle kept, as loading does), less the outflows
    launch_keys_from_positions(x->pa, x->n, x->c, x->keys, s);
    for (auto &src : x->sources)
        if (src.prm.enabled && !src.prm.inflow && src.prm.fluid_outflow)
            launch_outflow_mark(x->pa, x->n, x->c, src.dmask, src.prm.outflow_inversed ? 1 : 0, source_view(x, src),
                                x->keys, s);
    const int saveMax = x->maxPerCell;
    x->maxPerCell = 0x7fffffff;
    rc = rebin(x);
    x->maxPerCell = saveMax;
    return rc;
}

// Counting sort of the particles in `pa` by cell, with removal flags in
// keys; survivors land in `pb` ordered (cell, id); then the buffers swap.
int rebin(flip_ctx *x) {
    cudaStream_t s = x->stream;
    int nc = (int)x->nc();
    CK(cudaMemsetAsync(x->cellCount, 0, (size_t)(nc + 1) * sizeof(int), s));
    CK(cudaMemsetAsync(x->cursor, 0, (size_t)(nc + 1) * sizeof(int), s));
    CK(cudaMemsetAsync(x->maxVelSqBits, 0, sizeof(unsigned int), s));
    launch_bin_count(x->keys, x->n, x->cellCount, s);
    launch_scan_cells(x->cellCount, nc, x->cellStart, x->scanScratch, x->scanTotal, s);
    launch_bin_scatter(x->keys, x->n, x->cellStart, x->cursor, x->slots, s);
    launch_cell_sort_select(x->cellStart, nc, x->slots, x->pa.id, x->keys, x->maxPerCell, x->survivors, s);
    launch_scan_cells(x->survivors, nc, x->newStart, x->scanScratch, x->scanTotal, s);
    launch_gather_particles(x->pa, x->pb, x->cellStart, x->slots, x->newStart, nc, x->maxVelSqBits, s);
    CK(cudaMemcpyAsync(&x->mail->total, x->scanTotal, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&x->mail->velSqBits, x->maxVelSqBits, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
    if (x->endMarkPending) {
        x->mark(FLIP_NUM_STAGES);
        x->endMarkPending = false;
    }
    int rc = sync(x);
    if (rc) return rc;
    std::swap(x->pa, x->pb);
    std::swap(x->cellStart, x->newStart);
    x->n = x->mail->total;
    float vsq;
    std::memcpy(&vsq, &x->mail->velSqBits, 4);
    x->maxSpeed = std::sqrt((double)vsq);
    return FLIP_OK;
}

int rebin_marked(flip_ctx *x) {
    // rebin() synchronises; record the end mark before its final sync
    x->endMarkPending = true;
    return rebin(x);
}

int collect_stage_times(flip_ctx *x) {
    if (!x->timing) return FLIP_OK;
    FLIP_SYNC_COUNT();
    CK(cudaEventSynchronize(x->ev[FLIP_NUM_STAGES]));
    for (int q = 0; q < FLIP_NUM_STAGES; q++) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, x->ev[q], x->ev[q + 1]));
        x->stageMs[q] += ms;
    }
    x->timedSubsteps++;
    return FLIP_OK;
}

int build_solid(flip_ctx *x) {
    x->box.compute(x->I, x->J, x->K, x->dx, x->cfl, x->obstacles);
    cudaStream_t s = x->stream;
    CK(cudaMemcpyAsync(x->solidPhi, x->box.nodal.data(), x->box.nodal.size() * 4, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(x->wu, x->box.wu.data(), x->box.wu.size() * 4, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(x->wv, x->box.wv.data(), x->box.wv.size() * 4, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(x->ww, x->box.ww.data(), x->box.ww.size() * 4, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(x->solidCC, x->box.solidCentre.data(), x->box.solidCentre.size(), cudaMemcpyHostToDevice, s));
    int rc = x->nearSolid ? FLIP_OK : x->alloc(&x->nearSolid, x->box.near.size());
    if (rc) return rc;
    if (x->box.anyFriction) {
        if (!x->fu && ((rc = x->alloc(&x->fu, x->nu())) || (rc = x->alloc(&x->fv, x->nv())) ||
                       (rc = x->alloc(&x->fw, x->nw()))))
            return rc;
        CK(cudaMemcpyAsync(x->fu, x->box.fu.data(), x->box.fu.size() * 4, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(x->fv, x->box.fv.data(), x->box.fv.size() * 4, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(x->fw, x->box.fw.data(), x->box.fw.size() * 4, cudaMemcpyHostToDevice, s));
    }
    CK(cudaMemcpyAsync(x->nearSolid, x->box.near.data(), x->box.near.size(), cudaMemcpyHostToDevice, s));
    StepConsts &c = x->c;
    c.nsi = x->box.nsi; c.nsj = x->box.nsj; c.nsk = x->box.nsk;
    c.nearCell = x->box.nearCell;
    c.invNearCell = 1.0 / x->box.nearCell;
    c.invNearCellf = (float)c.invNearCell;
    // collision boundary: the domain box shrunk again by 0.1 dx
    double v2 = -((double)0.1f * x->dx), h2 = 0.5 * v2;
    c.bposx = x->box.px - (float)h2; c.bposy = x->box.py - (float)h2; c.bposz = x->box.pz - (float)h2;
    c.bw = x->box.ex + v2; c.bh = x->box.ey + v2; c.bd = x->box.ez + v2;
    rc = sync(x);
    if (rc) return rc;
    x->solidBuilt = true;
    return FLIP_OK;
}

template <class T>
void dl(flip_ctx *x, T *dst, const T *src, long long count) {
    if (dst) cudaMemcpyAsync(dst, src, count * sizeof(T), cudaMemcpyDeviceToHost, x->stream);
}

// Particles of the current arrays in the reference's order (by id).
// Particles [start, end) of the reference's order into host memory (packed
// xyz), reordered on the device: the idle particle buffer is the staging area.
int particles_to_host(flip_ctx *x, float *pos, float *vel, int start, int end) {
    int n = x->n;
    if (n == 0 || end <= start) return FLIP_OK;
    float *dpos = x->pb.px, *dvel = x->pb.px + 3 * (size_t)x->capacity;
    launch_readback_order(x->pa, n, x->idSpace, x->idFlags, x->idRank, x->idScratch, x->idTotal,
                          pos ? dpos : nullptr, vel ? dvel : nullptr, x->stream);
    size_t off = 3 * (size_t)start, bytes = 3 * (size_t)(end - start) * sizeof(float);
    if (pos) CK(cudaMemcpyAsync(pos, dpos + off, bytes, cudaMemcpyDeviceToHost, x->stream));
    if (vel) CK(cudaMemcpyAsync(vel, dvel + off, bytes, cudaMemcpyDeviceToHost, x->stream));
    return sync(x);
}

int particles_in_order(flip_ctx *x, std::vector<float> *pos, std::vector<float> *vel) {
    if (pos) pos->resize(3 * (size_t)x->n);
    if (vel) vel->resize(3 * (size_t)x->n);
    return particles_to_host(x, pos ? pos->data() : nullptr, vel ? vel->data() : nullptr, 0, x->n);
}

// PressureSolver::solve (pressuresolver.cpp:44-76) on the device: FLIP_OK
// when the velocities were updated or nothing needed solving,
// FLIP_E_SOLVER_NOCONV when the solve failed and they were left as they were.
int pressure_solve(flip_ctx *x, double dt, bool *applied, flip_stage_dump *d) {
    PressureArgs a;
    a.phi = x->phi; a.wu = x->wu; a.wv = x->wv; a.ww = x->ww;
    a.u = x->u; a.v = x->v; a.w = x->w;
    a.vu = x->vu; a.vv = x->vv; a.vw = x->vw;
    a.dt = dt; a.tol = x->tol; a.accTol = x->accTol; a.maxIter = x->maxIter;
    a.dumpPressure = d ? d->pressure : nullptr;
    a.dumpRhs = d ? d->rhs : nullptr;
    a.sweepTiming = x->timing ? &x->sweepTiming : nullptr;
    a.sweepOrientation = x->sweepOrientation;
    PressureResult res{};
    std::string msg;
    int rc = pressure_project(x->c, a, x->pr, x->sweep, x->pmail, x->stream, &res, &msg);
    x->stats.pressure_iterations = res.iterations;
    x->stats.pressure_error = res.residual;
    x->stats.pressure_cells = res.cells;
    *applied = res.applied;
    if (rc != FLIP_OK && rc != FLIP_E_SOLVER_NOCONV) return fail(rc, msg);
    return rc;
}

int dump_mac(flip_ctx *x, float *a, float *b, float *e, const float *u, const float *v, const float *w) {
    if (!a) return FLIP_OK;
    int rc = sync(x);
    if (rc) return rc;
    CK(cudaMemcpy(a, u, x->nu() * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(b, v, x->nv() * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(e, w, x->nw() * 4, cudaMemcpyDeviceToHost));
    return FLIP_OK;
}

// The viscosity solve's device buffers, made with the first viscous step.
int alloc_viscosity(flip_ctx *x) {
    if (x->vbReady) return FLIP_OK;
    long long nf, nn, ncorner, vol[7];
    int rb;
    viscosity_buffer_sizes(x->I, x->J, x->K, &nf, &nn, &ncorner, vol, &rb);
    ViscosityBuffers &b = x->vb;
    int rc;
    if ((rc = x->alloc(&b.fluidFace, nf)) || (rc = x->alloc(&b.valid, nn)) || (rc = x->alloc(&b.valid2, nn)) ||
        (rc = x->alloc(&b.inSys, nf)) || (rc = x->alloc(&b.node, ncorner)) || (rc = x->alloc(&b.fac, 2 * nf)) ||
        (rc = x->alloc(&b.dr, nf)) || (rc = x->alloc(&b.x, nf)) || (rc = x->alloc(&b.r, nf)) ||
        (rc = x->alloc(&b.z, nf)) || (rc = x->alloc(&b.p, nf)) || (rc = x->alloc(&b.q, nf)) ||
        (rc = x->alloc(&b.part, 3 * (long long)rb)) || (rc = x->alloc(&b.scal, 8)))
        return rc;
    for (int g = 0; g < 7; g++)
        if ((rc = x->alloc(&b.vol[g], vol[g]))) return rc;
    x->vbReady = true;
    return FLIP_OK;
}

// _applyViscosityToVelocityField (fluidsimulation.cpp:3592-3640): the field
// constrained first, then the viscosity solve (flip_viscosity.cu).
int apply_viscosity(flip_ctx *x, double dt) {
    x->viscResult = ViscosityResult{};
    if (!x->viscosityEnabled || x->n == 0 || !(x->viscosity > 0.0)) return FLIP_OK;
    int rc = alloc_viscosity(x);
    if (rc) return rc;
    const bool fr = x->box.anyFriction;
    launch_constrain(x->c, x->u, x->v, x->w, nullptr, nullptr, nullptr, x->wu, x->wv, x->ww, fr ? x->fu : nullptr,
                     fr ? x->fv : nullptr, fr ? x->fw : nullptr, x->stream);
    return viscosity_apply(x->c, x->vb, x->phi, x->solidPhi, x->u, x->v, x->w, x->viscosity, dt, &x->viscResult,
                           x->stream);
}

// _stepFluid (fluidsimulation.cpp:5471-5508)
// _updateForceFieldGrid (fluidsimulation.cpp:3440-3448) without adaptive
// force-field time stepping: at the first substep of a frame the grid takes
// the body force (a change of more than 1e-6 in length, ForceFieldGrid::
// setGravityVector, forcefieldgrid.cpp:103-110, or of a field rebuilds it);
// the grid's dimensions are ceil(I / level) ... at a cell of level * dx
// (_initializeForceFieldGrid, :2614-2621), fixed when it is first built.
int update_force_field_grid(flip_ctx *x, float3 bf) {
    if (x->stepNumber != 0 && x->ffU) return FLIP_OK;
    const float g[3] = {bf.x, bf.y, bf.z};
    const float dg[3] = {g[0] - x->ffGravity[0], g[1] - x->ffGravity[1], g[2] - x->ffGravity[2]};
    if (std::sqrt(dg[0] * dg[0] + dg[1] * dg[1] + dg[2] * dg[2]) > 1e-6f) x->ffDirty = true;
    for (int d = 0; d < 3; d++) x->ffGravity[d] = g[d];
    if (!x->ffDirty && x->ffU) return FLIP_OK;
    int rc;
    if (!x->ffU) {
        const int red = x->ffReduction;
        const int ni = (int)std::ceil((double)x->I / (double)red), nj = (int)std::ceil((double)x->J / (double)red),
                  nk = (int)std::ceil((double)x->K / (double)red);
        x->ffHost.ni = ni;
        x->ffHost.nj = nj;
        x->ffHost.nk = nk;
        x->ffHost.dx = x->dx * red;
        if ((rc = x->alloc(&x->ffU, (size_t)(ni + 1) * nj * nk)) || (rc = x->alloc(&x->ffV, (size_t)ni * (nj + 1) * nk)) ||
            (rc = x->alloc(&x->ffW, (size_t)ni * nj * (nk + 1))))
            return rc;
    }
    std::vector<PointForceField> fields;
    for (auto &e : x->forceFields) fields.push_back(e.f);
    point_force_grid(x->ffHost.ni, x->ffHost.nj, x->ffHost.nk, x->ffHost.dx, fields, g, x->ffHost);
    CK(cudaMemcpyAsync(x->ffU, x->ffHost.u.data(), x->ffHost.u.size() * 4, cudaMemcpyHostToDevice, x->stream));
    CK(cudaMemcpyAsync(x->ffV, x->ffHost.v.data(), x->ffHost.v.size() * 4, cudaMemcpyHostToDevice, x->stream));
    CK(cudaMemcpyAsync(x->ffW, x->ffHost.w.data(), x->ffHost.w.size() * 4, cudaMemcpyHostToDevice, x->stream));
    x->ffDirty = false;
    return FLIP_OK;
}

int step_fluid(flip_ctx *x, double dt, flip_stage_dump *d) {
    cudaStream_t s = x->stream;
    StepConsts &c = x->c;
    int rc;
    if (d && d->n_before) *d->n_before = x->n;
    if (!x->solidBuilt && x->n > 0) {
        if ((rc = build_solid(x))) return rc;
    }
    int layers = (int)std::ceil(x->cfl) + 2;
    x->mark(FLIP_STAGE_LIQUID_SDF);
    // liquid level set (particlelevelset.cpp:161-196)
    if (x->n > 0 && x->solidBuilt) {
        launch_liquid_sdf(x->pa, x->cellStart, c, x->solidCC, x->phi, x->sdfThreads, s);
    } else {
        std::vector<float> fill(x->nc(), (float)(3.0 * x->dx));
        float eps = (float)(0.005 * x->dx);
        for (auto &f : fill) if (std::abs(f) < eps) f = f > 0 ? eps : -eps;
        CK(cudaMemcpyAsync(x->phi, fill.data(), fill.size() * 4, cudaMemcpyHostToDevice, s));
        FLIP_SYNC_COUNT();
        CK(cudaStreamSynchronize(s));
    }
    if (d && d->phi) {
        if ((rc = sync(x))) return rc;
        CK(cudaMemcpy(d->phi, x->phi, x->nc() * 4, cudaMemcpyDeviceToHost));
    }
    // advect velocity field: P2G + extrapolation (fluidsimulation.cpp:3253-3285)
    x->mark(FLIP_STAGE_P2G);
    if (x->n > 0) {
        launch_p2g(x->pa, x->cellStart, c, x->u, x->v, x->w, x->vu, x->vv, x->vw, s);
        if (d && d->vu_p2g) {
            if ((rc = sync(x))) return rc;
            CK(cudaMemcpy(d->vu_p2g, x->vu, x->nu(), cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(d->vv_p2g, x->vv, x->nv(), cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(d->vw_p2g, x->vw, x->nw(), cudaMemcpyDeviceToHost));
        }
        launch_extrapolate(c, x->u, x->v, x->w, x->vu, x->vv, x->vw, x->status, layers, s);
    } else {
        CK(cudaMemsetAsync(x->u, 0, x->nu() * 4, s));
        CK(cudaMemsetAsync(x->v, 0, x->nv() * 4, s));
        CK(cudaMemsetAsync(x->w, 0, x->nw() * 4, s));
        CK(cudaMemsetAsync(x->vu, 0, x->nu(), s));
        CK(cudaMemsetAsync(x->vv, 0, x->nv(), s));
        CK(cudaMemsetAsync(x->vw, 0, x->nw(), s));
    }
    if (d && (rc = dump_mac(x, d->u_p2g, d->v_p2g, d->w_p2g, x->u, x->v, x->w))) return rc;
    // save + constant body force (fluidsimulation.cpp:3287-3297, 3450-3489)
    x->mark(FLIP_STAGE_FORCE);
    float3 bf = body_force(x);
    const float feps = 1e-6f;
    // inflow sources that constrain the fluid velocity keep the force off their faces
    InflowConstraint ic;
    if ((rc = inflow_constraint(x, &ic))) return rc;
    if (ic.count) launch_inflow_faces(c, ic, x->vu, x->vv, x->vw, x->inflowFaces, s);
    if (x->ffEnabled) {
        // _applyBodyForcesToVelocityField with force fields (:3566-3583):
        // save, then the force-field grid instead of the constant force
        if ((rc = update_force_field_grid(x, bf))) return rc;
        launch_save_and_force(c, x->u, x->v, x->w, x->su, x->sv, x->sw, 0.f, 0.f, 0.f, false, false, false, nullptr, s);
        ForceFieldView fv{x->ffU, x->ffV, x->ffW, x->ffHost.ni, x->ffHost.nj, x->ffHost.nk, x->ffHost.dx,
                          x->ffGravity[0], x->ffGravity[1], x->ffGravity[2]};
        launch_force_field(c, x->u, x->v, x->w, fv, dt, ic.count ? x->inflowFaces : nullptr, s);
    } else {
        launch_save_and_force(c, x->u, x->v, x->w, x->su, x->sv, x->sw, (float)(bf.x * dt), (float)(bf.y * dt),
                              (float)(bf.z * dt), std::fabs(bf.x) > feps, std::fabs(bf.y) > feps,
                              std::fabs(bf.z) > feps, ic.count ? x->inflowFaces : nullptr, s);
    }
    if (d && (rc = dump_mac(x, d->u_force, d->v_force, d->w_force, x->u, x->v, x->w))) return rc;
    if ((rc = apply_viscosity(x, dt))) return rc;
    // pressure (fluidsimulation.cpp:3732-3773)
    if (!x->solidBuilt) {
        if ((rc = build_solid(x))) return rc;
    }
    bool applied = false;
    x->mark(FLIP_STAGE_PRESSURE);
    rc = pressure_solve(x, dt, &applied, d);
    if (rc != FLIP_OK && rc != FLIP_E_SOLVER_NOCONV) return rc;
    x->stats.pressure_status = rc;
    if (d && d->pcg_iters) *d->pcg_iters = x->stats.pressure_iterations;
    if (d && d->pcg_error) *d->pcg_error = x->stats.pressure_error;
    x->mark(FLIP_STAGE_CONSTRAIN);
    launch_extrapolate(c, x->u, x->v, x->w, x->vu, x->vv, x->vw, x->status, layers, s);
    if (d && (rc = dump_mac(x, d->u_press, d->v_press, d->w_press, x->u, x->v, x->w))) return rc;
    // constrain saved and current fields (fluidsimulation.cpp:3937-3950)
    const bool fr = x->box.anyFriction;
    launch_constrain(c, x->u, x->v, x->w, x->su, x->sv, x->sw, x->wu, x->wv, x->ww, fr ? x->fu : nullptr,
                     fr ? x->fv : nullptr, fr ? x->fw : nullptr, s);
    if (d && (rc = dump_mac(x, d->u_final, d->v_final, d->w_final, x->u, x->v, x->w))) return rc;
    if (d && (rc = dump_mac(x, d->u_saved, d->v_saved, d->w_saved, x->su, x->sv, x->sw))) return rc;
    if (x->n == 0) {
        x->mark(FLIP_STAGE_ADVECT);
        x->mark(FLIP_STAGE_BINNING);
        x->mark(FLIP_NUM_STAGES);
        if ((rc = collect_stage_times(x))) return rc;
        return update_fluid_objects(x);   // _updateFluidObjects (fluidsimulation.cpp:5505)
    }
    // particle velocities, advection, removal (fluidsimulation.cpp:4172-4390)
    x->mark(FLIP_STAGE_ADVECT);
    double speedStep = x->cfl * x->dx / x->frameDt;
    CK(cudaMemsetAsync(x->speedHist, 0, 8 * sizeof(unsigned int), s));
    launch_advect(x->pa, x->n, c, x->u, x->v, x->w, x->su, x->sv, x->sw, x->solidPhi, x->nearSolid,
                  (float)x->picRatio, (float)(1 - x->picRatio), dt, x->keys, x->speedHist, speedStep, ic, s);
    if (d && (d->vel_g2p || d->pos_adv)) {
        std::vector<float> pos, vel;
        if ((rc = particles_in_order(x, &pos, &vel))) return rc;
        if (d->vel_g2p) std::memcpy(d->vel_g2p, vel.data(), vel.size() * 4);
        if (d->pos_adv) std::memcpy(d->pos_adv, pos.data(), pos.size() * 4);
    }
    launch_speed_limit(x->speedHist, x->n, x->maxFrameSteps, speedStep, x->maxRemovePct, x->maxRemoveAbs,
                       x->maxSpeedSq, s);
    launch_mark_fast(x->pa, x->n, x->maxSpeedSq, x->keys, s);
    x->mark(FLIP_STAGE_BINNING);
    rc = rebin_marked(x);
    if (rc) return rc;
    if ((rc = collect_stage_times(x))) return rc;
    return update_fluid_objects(x);   // _updateFluidObjects (fluidsimulation.cpp:5505)
}

// The surface mesh of the current particles (_launchOutputSurfaceMeshThread
// and _outputSurfaceMeshThread, fluidsimulation.cpp:5150-5239): radius =
// marker particle radius (_initializeParticleRadii, :2643-2649) x marker
// particle scale; the solid level set as the step uses it.
int build_isomesh(flip_ctx *x) {
    MeshJob job{};
    job.c = x->c;
    job.p = x->pa;
    job.n = x->n;
    job.cellStart = x->cellStart;
    job.solidPhi = x->solidPhi;
    job.subdivisions = x->meshSubdivisions;
    const double volume = x->dx * x->dx * x->dx / 8.0, pi = 3.141592653;
    job.radius = std::pow(3 * volume / (4 * pi), 1.0 / 3.0) * x->markerParticleScale;
    job.smoothValue = x->meshSmoothValue;
    job.smoothIterations = x->meshSmoothIterations;
    if (x->n > 0 && !x->solidBuilt) {
        int rc = build_solid(x);
        if (rc) return rc;
    }
    return mesh_surface(job, x->mesh, x->stream);
}

// _calculateNextTimeStep (fluidsimulation.cpp:5593-5613)
double next_time_step(flip_ctx *x, double dt) {
    double maxu;
    if (x->frame == 0 && x->stepNumber == 0) {
        // _predictMaximumMarkerParticleSpeed (:5529-5550): the queued fluid
        // meshes' speeds, plus the body force over one frame
        maxu = 0.0;
        for (const auto &fm : x->fluidQueue)
            maxu = std::fmax((double)std::sqrt(fm.vx * fm.vx + fm.vy * fm.vy + fm.vz * fm.vz), maxu);
        for (const auto &src : x->sources) {   // enabled inflow sources (:5537-5546)
            if (!src.prm.enabled || !src.prm.inflow) continue;
            const float vx = (float)src.prm.velocity[0], vy = (float)src.prm.velocity[1], vz = (float)src.prm.velocity[2];
            maxu = std::fmax((double)std::sqrt(vx * vx + vy * vy + vz * vz), maxu);
        }
        float3 bf = body_force(x);
        float len = std::sqrt(bf.x * bf.x + bf.y * bf.y + bf.z * bf.z);
        maxu += len * dt;
    } else {
        maxu = x->maxSpeed;
    }
    maxu = std::fmax(0.0, maxu);
    return x->cfl * x->dx / (maxu + 1e-6);
}

int do_update(flip_ctx *x, double dt, flip_stage_dump *d) {
    if (!x->initialized) return fail(FLIP_E_RUNTIME, "Error: FluidSimulation must be initialized before update.");
    if (dt < 0.0) return fail(FLIP_E_DOMAIN, "Error: delta time must be greater than or equal to 0.");
    double epsdt = 1e-6;
    bool zeroLength = dt < epsdt;
    dt = std::max(dt, epsdt);
    x->frameDt = dt;
    x->frameRemaining = dt;
    x->stepNumber = 0;
    bool skipped = zeroLength && x->outputInitialized;
    double substep = dt / (double)x->minFrameSteps;
    double eps = 1e-9;
    int worst = FLIP_OK;
    do {
        double step = std::fmin(next_time_step(x, dt), x->frameRemaining);
        if (d && step < dt) return fail(FLIP_E_RUNTIME, "staged update: the frame needs more than one substep");
        double done = x->frameDt - x->frameRemaining;
        double limit = (x->stepNumber + 1) * substep;
        if (done + step > limit) step = std::fmin(substep, x->frameRemaining);
        if (x->stepNumber == x->maxFrameSteps - 1) step = x->frameRemaining;
        x->frameRemaining -= step;
        if (!skipped) {
            int rc = step_fluid(x, step, d);
            if (rc == FLIP_E_SOLVER_NOCONV) worst = rc;
            else if (rc != FLIP_OK) return rc;
            if (x->stats.pressure_status == FLIP_E_SOLVER_NOCONV) worst = FLIP_E_SOLVER_NOCONV;
            // _outputSimulationData (fluidsimulation.cpp:5444-5464): the
            // frame's mesh comes from the state after its first substep
            if (x->stepNumber == 0 && x->meshEnabled && (rc = build_isomesh(x))) return rc;
        }
        d = nullptr;
        x->stepNumber++;
    } while (x->frameRemaining > eps);
    x->stats.frame = x->frame;
    x->stats.substeps = x->stepNumber;
    x->stats.delta_time = dt;
    x->stats.fluid_particles = x->n;
    x->stats.pressure_status = worst;
    x->outputInitialized = true;
    x->frame++;
    return FLIP_OK;
}

int do_initialize(flip_ctx *x) {
    if (x->initialized) return FLIP_OK;
    cudaStream_t s = x->stream;
    int rc;
    // _loadMarkerParticles (fluidsimulation.cpp:2773-2786): keep points in
    // [0, I dx) x [0, J dx) x [0, K dx)
    std::vector<float> hp, hv;
    if (x->queueDevN > 0) {
        hp.resize(3 * (size_t)x->queueDevN);
        hv.resize(3 * (size_t)x->queueDevN);
        CK(cudaMemcpy(hp.data(), x->queueDevPos, hp.size() * 4, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(hv.data(), x->queueDevVel, hv.size() * 4, cudaMemcpyDeviceToHost));
    }
    hp.insert(hp.begin(), x->queuePos.begin(), x->queuePos.end());
    hv.insert(hv.begin(), x->queueVel.begin(), x->queueVel.end());
    double W = x->I * x->dx, H = x->J * x->dx, D = x->K * x->dx;
    int total = (int)(hp.size() / 3);
    std::vector<float> sx, sy, sz, svx, svy, svz;
    for (int q = 0; q < total; q++) {
        float a = hp[3 * q] * 1.0f, b = hp[3 * q + 1] * 1.0f, e = hp[3 * q + 2] * 1.0f;
        if (a >= 0.0f && b >= 0.0f && e >= 0.0f && a < 0.0 + W && b < 0.0 + H && e < 0.0 + D) {
            sx.push_back(a); sy.push_back(b); sz.push_back(e);
            svx.push_back(hv[3 * q]); svy.push_back(hv[3 * q + 1]); svz.push_back(hv[3 * q + 2]);
        }
    }
    x->queuePos.clear(); x->queueVel.clear(); x->queueDevN = 0;
    x->n = (int)sx.size();
    x->idNext = (unsigned int)x->n;
    if ((rc = alloc_particles(x, std::max(x->n, 1)))) return rc;
    if (x->n > 0) {
        std::vector<unsigned int> ids(x->n);
        for (int q = 0; q < x->n; q++) ids[q] = (unsigned int)q;
        CK(cudaMemcpyAsync(x->pa.px, sx.data(), x->n * 4, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(x->pa.py, sy.data(), x->n * 4, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(x->pa.pz, sz.data(), x->n * 4, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(x->pa.vx, svx.data(), x->n * 4, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(x->pa.vy, svy.data(), x->n * 4, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(x->pa.vz, svz.data(), x->n * 4, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(x->pa.id, ids.data(), x->n * 4, cudaMemcpyHostToDevice, s));
        launch_keys_from_positions(x->pa, x->n, x->c, x->keys, s);
        int saveMax = x->maxPerCell;
        x->maxPerCell = 0x7fffffff;          // loading keeps every particle
        rc = rebin(x);
        x->maxPerCell = saveMax;
        if (rc) return rc;
    } else {
        CK(cudaMemsetAsync(x->cellStart, 0, (x->nc() + 1) * sizeof(int), s));
    }
    x->initialized = true;
    // the static solid set-up, as the reference makes it on initialisation
    // (it is redone before the next step if an obstacle or the CFL number
    // changes)
    if (!x->solidBuilt && (rc = build_solid(x))) return rc;
    return sync(x);
}

}  // namespace

namespace flip {
int record_error(int code, const std::string &msg) { return fail(code, msg); }
}  // namespace flip

// ====================================================================== C ABI
extern "C" {

const char *flip_last_error(void) { return g_err.c_str(); }

int flip_create(int isize, int jsize, int ksize, double dx, flip_ctx **out) {
    if (!out) return fail(FLIP_E_NULL, "null output pointer");
    *out = nullptr;
    if (isize <= 0 || jsize <= 0 || ksize <= 0 || !(dx > 0.0))
        return fail(FLIP_E_DOMAIN, "Error: dimensions and cell size must be greater than 0.");
    if ((long long)isize * jsize * ksize >= (1LL << 28))
        return fail(FLIP_E_DOMAIN, "grid too large for 28-bit cell keys");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail(FLIP_E_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    flip_ctx *x = new flip_ctx();
    x->I = isize; x->J = jsize; x->K = ksize; x->dx = dx;
    cudaGetDevice(&x->device);
    if (cudaStreamCreateWithFlags(&x->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete x;
        return fail(FLIP_E_CUDA, "cudaStreamCreate failed");
    }
    x->ownStream = true;
    if (cudaMallocHost((void **)&x->mail, sizeof(flip_ctx::Mail)) != cudaSuccess ||
        cudaMallocHost((void **)&x->pmail, sizeof(PressureMail)) != cudaSuccess) {
        cudaStreamDestroy(x->stream);
        delete x;
        return fail(FLIP_E_NOMEM, "cudaMallocHost failed");
    }
    StepConsts &c = x->c;
    c.I = isize; c.J = jsize; c.K = ksize;
    c.dx = dx; c.invdx = 1.0 / dx; c.invdxf = (float)(1.0 / dx); c.dxf = (float)dx;
    c.radius = 0.5 * 1.0 * dx * std::sqrt(3.0);
    auto below = [](double bound) {   // largest float v with (double)v < bound
        float v = (float)bound;
        while ((double)v >= bound) v = std::nextafter(v, 0.0f);
        return v;
    };
    c.gxmax = below(dx * isize);
    c.gymax = below(dx * jsize);
    c.gzmax = below(dx * ksize);
    c.cfl = x->cfl;
    c.maxPerCell = x->maxPerCell;
    int rc = alloc_grids(x);
    if (rc) {
        flip_destroy(x);
        return rc;
    }
    *out = x;
    return FLIP_OK;
}

int flip_destroy(flip_ctx *x) {
    if (!x) return FLIP_E_NULL;
    FLIP_SYNC_COUNT();
    cudaStreamSynchronize(x->stream);
    for (int q = 0; q < 2; q++)   // the graphs refer to the timing events: first
        for (int o = 0; o < 2; o++)
            if (x->pr.batchGraph[q][o]) cudaGraphExecDestroy(x->pr.batchGraph[q][o]);
    for (int o = 0; o < 2; o++)
        if (x->pr.loopGraph[o]) cudaGraphExecDestroy(x->pr.loopGraph[o]);
    for (int q = 0; q <= FLIP_NUM_STAGES; q++)
        if (x->ev[q]) cudaEventDestroy(x->ev[q]);
    for (int q = 0; q < 2 * (PCG_BATCH + 1); q++)
        if (x->sweepTiming.ev[q]) cudaEventDestroy(x->sweepTiming.ev[q]);
    for (void *p : x->allocations) cudaFree(p);
    mesh_release(x->mesh);
    if (x->mail) cudaFreeHost(x->mail);
    if (x->pmail) cudaFreeHost(x->pmail);
    if (x->ownStream) cudaStreamDestroy(x->stream);
    delete x;
    return FLIP_OK;
}

int flip_set_stream(flip_ctx *x, void *stream) {
    if (!x) return FLIP_E_NULL;
    FLIP_SYNC_COUNT();
    cudaStreamSynchronize(x->stream);
    if (stream) {
        if (x->ownStream) cudaStreamDestroy(x->stream);
        x->stream = (cudaStream_t)stream;
        x->ownStream = false;
    }
    return FLIP_OK;
}

int flip_set_pic_flip_ratio(flip_ctx *x, double r) {
    if (!x) return FLIP_E_NULL;
    if (r < 0.0 || r > 1.0) return fail(FLIP_E_DOMAIN, "Error: PICFLIP ratio must be in range [0.0, 1.0].");
    x->picRatio = r;
    return FLIP_OK;
}
int flip_get_pic_flip_ratio(flip_ctx *x, double *r) {
    if (!x || !r) return FLIP_E_NULL;
    *r = x->picRatio;
    return FLIP_OK;
}
int flip_add_body_force(flip_ctx *x, double fx, double fy, double fz) {
    if (!x) return FLIP_E_NULL;
    x->bodyForces.push_back((float)fx);
    x->bodyForces.push_back((float)fy);
    x->bodyForces.push_back((float)fz);
    return FLIP_OK;
}
int flip_reset_body_force(flip_ctx *x) {
    if (!x) return FLIP_E_NULL;
    x->bodyForces.clear();
    return FLIP_OK;
}
int flip_set_cfl_condition_number(flip_ctx *x, int n) {
    if (!x) return FLIP_E_NULL;
    if (n < 1) return fail(FLIP_E_DOMAIN, "Error: CFL must be greater than or equal to 1.");
    if (x->outputInitialized) return fail(FLIP_E_RUNTIME, "CFL number is fixed once the simulation has stepped");
    if (n != (int)x->cfl) x->solidBuilt = false;   // the near-solid grid depends on it
    x->cfl = n;
    x->c.cfl = n;
    return FLIP_OK;
}
int flip_set_pressure_tolerance(flip_ctx *x, double tol) {
    if (!x) return FLIP_E_NULL;
    if (!(tol > 0.0)) return fail(FLIP_E_DOMAIN, "tolerance must be positive");
    x->tol = tol;
    return FLIP_OK;
}
int flip_set_max_pressure_iterations(flip_ctx *x, int n) {
    if (!x) return FLIP_E_NULL;
    if (n < 1) return fail(FLIP_E_DOMAIN, "iterations must be positive");
    x->maxIter = n;
    return FLIP_OK;
}
int flip_load_marker_particle_data(flip_ctx *x, int n, const float *pos, const float *vel) {
    if (!x) return FLIP_E_NULL;
    LaunchTally tally(x);
    if (n < 0) return fail(FLIP_E_DOMAIN, "negative particle count");
    if (n == 0) return FLIP_OK;
    if (!pos || !vel) return FLIP_E_NULL;
    if (x->initialized) return fail(FLIP_E_RUNTIME, "particles are loaded before initialize()");
    x->queuePos.insert(x->queuePos.end(), pos, pos + 3 * (size_t)n);
    x->queueVel.insert(x->queueVel.end(), vel, vel + 3 * (size_t)n);
    return FLIP_OK;
}
int flip_load_marker_particle_data_device(flip_ctx *x, int n, const float *dpos, const float *dvel) {
    if (!x) return FLIP_E_NULL;
    LaunchTally tally(x);
    if (n < 0) return fail(FLIP_E_DOMAIN, "negative particle count");
    if (n == 0) return FLIP_OK;
    if (!dpos || !dvel) return FLIP_E_NULL;
    if (x->initialized) return fail(FLIP_E_RUNTIME, "particles are loaded before initialize()");
    if (x->queueDevN) return fail(FLIP_E_RUNTIME, "one device particle load per simulation");
    x->queueDevPos = dpos; x->queueDevVel = dvel; x->queueDevN = n;
    return FLIP_OK;
}
int flip_initialize(flip_ctx *x) {
    if (!x) return FLIP_E_NULL;
    LaunchTally tally(x);
    return do_initialize(x);
}
int flip_is_initialized(flip_ctx *x, int *yes) {
    if (!x || !yes) return FLIP_E_NULL;
    *yes = x->initialized ? 1 : 0;
    return FLIP_OK;
}
int flip_update(flip_ctx *x, double dt) {
    if (!x) return FLIP_E_NULL;
    LaunchTally tally(x);
    return do_update(x, dt, nullptr);
}
int flip_update_staged(flip_ctx *x, double dt, flip_stage_dump *d) {
    if (!x || !d) return FLIP_E_NULL;
    LaunchTally tally(x);
    return do_update(x, dt, d);
}
int flip_get_num_marker_particles(flip_ctx *x, int *n) {
    if (!x || !n) return FLIP_E_NULL;
    *n = x->n;
    return FLIP_OK;
}
int flip_get_marker_particle_position_data(flip_ctx *x, float *out) {
    if (!x || !out) return FLIP_E_NULL;
    LaunchTally tally(x);
    return particles_to_host(x, out, nullptr, 0, x->n);
}
int flip_get_marker_particle_velocity_data(flip_ctx *x, float *out) {
    if (!x || !out) return FLIP_E_NULL;
    LaunchTally tally(x);
    return particles_to_host(x, nullptr, out, 0, x->n);
}
static int range_get(flip_ctx *x, int start, int end, float *out, bool vel) {
    if (!x || !out) return FLIP_E_NULL;
    if (start < 0 || end > x->n || start > end) return fail(FLIP_E_DOMAIN, "Error: invalid range.");
    return vel ? particles_to_host(x, nullptr, out, start, end) : particles_to_host(x, out, nullptr, start, end);
}
int flip_get_marker_particle_position_data_range(flip_ctx *x, int start, int end, float *out) {
    LaunchTally tally(x);
    return range_get(x, start, end, out, false);
}
int flip_get_marker_particle_velocity_data_range(flip_ctx *x, int start, int end, float *out) {
    LaunchTally tally(x);
    return range_get(x, start, end, out, true);
}
int flip_get_marker_particle_data_device(flip_ctx *x, float *dpos, float *dvel) {
    if (!x) return FLIP_E_NULL;
    cudaStream_t s = x->stream;
    int n = x->n;
    if (dpos) {
        CK(cudaMemcpyAsync(dpos, x->pa.px, n * 4, cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(dpos + n, x->pa.py, n * 4, cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(dpos + 2 * (size_t)n, x->pa.pz, n * 4, cudaMemcpyDeviceToDevice, s));
    }
    if (dvel) {
        CK(cudaMemcpyAsync(dvel, x->pa.vx, n * 4, cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(dvel + n, x->pa.vy, n * 4, cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(dvel + 2 * (size_t)n, x->pa.vz, n * 4, cudaMemcpyDeviceToDevice, s));
    }
    return FLIP_OK;
}
int flip_get_frame_stats(flip_ctx *x, flip_frame_stats *out) {
    if (!x || !out) return FLIP_E_NULL;
    *out = x->stats;
    return FLIP_OK;
}
int flip_get_current_frame(flip_ctx *x, int *frame) {
    if (!x || !frame) return FLIP_E_NULL;
    *frame = x->frame;
    return FLIP_OK;
}
int flip_get_binned_particles(flip_ctx *x, float *pos, unsigned int *ids, int *cell_start) {
    if (!x) return FLIP_E_NULL;
    int rc = sync(x);
    if (rc) return rc;
    const size_t n = (size_t)x->n;
    if (pos && n) {
        CK(cudaMemcpy(pos, x->pa.px, n * 4, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(pos + n, x->pa.py, n * 4, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(pos + 2 * n, x->pa.pz, n * 4, cudaMemcpyDeviceToHost));
    }
    if (ids && n) CK(cudaMemcpy(ids, x->pa.id, n * 4, cudaMemcpyDeviceToHost));
    if (cell_start) CK(cudaMemcpy(cell_start, x->cellStart, (x->nc() + 1) * sizeof(int), cudaMemcpyDeviceToHost));
    return FLIP_OK;
}
int flip_set_device_wait_limit(flip_ctx *x, unsigned int polls) {
    if (!x) return FLIP_E_NULL;
    x->sweep.spinLimit = polls;
    return FLIP_OK;
}
int flip_inject_sweep_stall(flip_ctx *x, int on) {
    if (!x) return FLIP_E_NULL;
    x->sweep.stall = on ? 1 : 0;
    return FLIP_OK;
}
int flip_set_current_frame(flip_ctx *x, int frame) {
    if (!x) return FLIP_E_NULL;
    if (frame < 0) return fail(FLIP_E_DOMAIN, "Error: frame number must be greater than or equal to 0.");
    x->frame = frame;
    return FLIP_OK;
}
int flip_get_liquid_sdf(flip_ctx *x, float *phi) {
    if (!x || !phi) return FLIP_E_NULL;
    int rc = sync(x);
    if (rc) return rc;
    CK(cudaMemcpy(phi, x->phi, x->nc() * 4, cudaMemcpyDeviceToHost));
    return FLIP_OK;
}
int flip_get_solid_sdf(flip_ctx *x, float *nodal) {
    if (!x || !nodal) return FLIP_E_NULL;
    if (!x->solidBuilt) {
        int rc = build_solid(x);
        if (rc) return rc;
    }
    std::memcpy(nodal, x->box.nodal.data(), x->box.nodal.size() * 4);
    return FLIP_OK;
}
int flip_get_mac_velocity(flip_ctx *x, float *u, float *v, float *w) {
    if (!x || !u || !v || !w) return FLIP_E_NULL;
    return dump_mac(x, u, v, w, x->u, x->v, x->w);
}
int flip_get_face_weights(flip_ctx *x, float *wu, float *wv, float *ww) {
    if (!x || !wu || !wv || !ww) return FLIP_E_NULL;
    if (!x->solidBuilt) {
        int rc = build_solid(x);
        if (rc) return rc;
    }
    std::memcpy(wu, x->box.wu.data(), x->box.wu.size() * 4);
    std::memcpy(wv, x->box.wv.data(), x->box.wv.size() * 4);
    std::memcpy(ww, x->box.ww.data(), x->box.ww.size() * 4);
    return FLIP_OK;
}
namespace {
// Obstacles given as plain arrays: obstacle q has nverts[q] vertices (xyz,
// consecutive in verts) and ntris[q] triangles (vertex indices local to it,
// consecutive in tris).
int obstacles_from_arrays(int n, const int *nverts, const float *verts, const int *ntris, const int *tris,
                          const float *friction, std::vector<MeshObstacle> &out) {
    if (n < 0) return fail(FLIP_E_DOMAIN, "negative obstacle count");
    if (n > 0 && (!nverts || !verts || !ntris || !tris)) return fail(FLIP_E_NULL, "null obstacle array");
    size_t vo = 0, to = 0;
    for (int q = 0; q < n; q++) {
        if (nverts[q] < 0 || ntris[q] < 0) return fail(FLIP_E_DOMAIN, "negative vertex or triangle count");
        MeshObstacle m;
        m.verts.assign(verts + 3 * vo, verts + 3 * (vo + nverts[q]));
        m.tris.assign(tris + 3 * to, tris + 3 * (to + ntris[q]));
        for (int t : m.tris)
            if (t < 0 || t >= nverts[q]) return fail(FLIP_E_DOMAIN, "triangle vertex index out of range");
        for (float v : m.verts)
            if (!std::isfinite(v)) return fail(FLIP_E_DOMAIN, "non-finite obstacle vertex");
        m.friction = friction ? friction[q] : 0.0f;
        if (!(m.friction >= 0.0f && m.friction <= 1.0f)) return fail(FLIP_E_DOMAIN, "friction must be in [0, 1]");
        vo += nverts[q];
        to += ntris[q];
        out.push_back(std::move(m));
    }
    return FLIP_OK;
}
}  // namespace

int flip_add_mesh_obstacle(flip_ctx *x, int nverts, const float *verts, int ntris, const int *tris, float friction) {
    if (!x) return FLIP_E_NULL;
    std::vector<MeshObstacle> one;
    int rc = obstacles_from_arrays(1, &nverts, verts, &ntris, tris, &friction, one);
    if (rc) return rc;
    x->obstacles.push_back(std::move(one[0]));
    x->solidBuilt = false;   // rebuilt before the next step (_isSolidLevelSetUpToDate, fluidsimulation.cpp:2007)
    return FLIP_OK;
}

int flip_add_mesh_fluid(flip_ctx *x, int nverts, const float *verts, int ntris, const int *tris, double vx, double vy,
                        double vz) {
    if (!x) return FLIP_E_NULL;
    std::vector<MeshObstacle> one;   // the same checks as an obstacle's arrays
    int rc = obstacles_from_arrays(1, &nverts, verts, &ntris, tris, nullptr, one);
    if (rc) return rc;
    if (!std::isfinite(vx) || !std::isfinite(vy) || !std::isfinite(vz)) return fail(FLIP_E_DOMAIN, "non-finite velocity");
    flip_ctx::FluidMesh fm;
    fm.verts = std::move(one[0].verts);
    fm.tris = std::move(one[0].tris);
    fm.vx = (float)vx; fm.vy = (float)vy; fm.vz = (float)vz;   // vmath::vec3
    x->fluidQueue.push_back(std::move(fm));
    return FLIP_OK;
}

int flip_set_marker_particle_jitter_factor(flip_ctx *x, double jit) {
    if (!x) return FLIP_E_NULL;
    if (!(jit >= 0.0)) return fail(FLIP_E_DOMAIN, "Error: marker particle jitter must be greater than or equal to 0.");
    x->jitterFactor = jit;
    return FLIP_OK;
}
int flip_get_marker_particle_jitter_factor(flip_ctx *x, double *jit) {
    if (!x || !jit) return FLIP_E_NULL;
    *jit = x->jitterFactor;
    return FLIP_OK;
}
int flip_set_jitter_surface_marker_particles(flip_ctx *x, int enable) {
    if (!x) return FLIP_E_NULL;
    x->jitterSurface = enable != 0;
    return FLIP_OK;
}
int flip_is_jitter_surface_marker_particles_enabled(flip_ctx *x, int *enabled) {
    if (!x || !enabled) return FLIP_E_NULL;
    *enabled = x->jitterSurface ? 1 : 0;
    return FLIP_OK;
}

int flip_mesh_fluid_cells(int isize, int jsize, int ksize, double dx, int nverts, const float *verts, int ntris,
                          const int *tris, int *ncells, int *cells, float *phi) {
    if (!ncells) return FLIP_E_NULL;
    if (isize <= 0 || jsize <= 0 || ksize <= 0 || !(dx > 0.0)) return fail(FLIP_E_DOMAIN, "bad grid");
    std::vector<MeshObstacle> one;
    int rc = obstacles_from_arrays(1, &nverts, verts, &ntris, tris, nullptr, one);
    if (rc) return rc;
    std::vector<int> c;
    std::vector<float> p;
    mesh_fluid_cells(isize, jsize, ksize, dx, one[0].verts, one[0].tris, c, p);
    *ncells = (int)c.size();
    if (cells) std::copy(c.begin(), c.end(), cells);
    if (phi) std::copy(p.begin(), p.end(), phi);
    return FLIP_OK;
}

int flip_compute_solid(int isize, int jsize, int ksize, double dx, int cfl, int nobstacles, const int *nverts,
                       const float *verts, const int *ntris, const int *tris, const float *friction, float *nodal,
                       float *wu, float *wv, float *ww, int *nearDims, uint8_t *nearOut, float *fu, float *fv,
                       float *fw) {
    if (isize <= 0 || jsize <= 0 || ksize <= 0 || !(dx > 0.0) || cfl < 1)
        return fail(FLIP_E_DOMAIN, "bad grid or CFL number");
    std::vector<MeshObstacle> obs;
    int rc = obstacles_from_arrays(nobstacles, nverts, verts, ntris, tris, friction, obs);
    if (rc) return rc;
    DomainBox b;
    b.compute(isize, jsize, ksize, dx, cfl, obs);
    if (nodal) std::memcpy(nodal, b.nodal.data(), b.nodal.size() * 4);
    if (wu) std::memcpy(wu, b.wu.data(), b.wu.size() * 4);
    if (wv) std::memcpy(wv, b.wv.data(), b.wv.size() * 4);
    if (ww) std::memcpy(ww, b.ww.data(), b.ww.size() * 4);
    if (nearDims) { nearDims[0] = b.nsi; nearDims[1] = b.nsj; nearDims[2] = b.nsk; }
    if (nearOut) std::memcpy(nearOut, b.near.data(), b.near.size());
    if (fu) std::memcpy(fu, b.fu.data(), b.fu.size() * 4);
    if (fv) std::memcpy(fv, b.fv.data(), b.fv.size() * 4);
    if (fw) std::memcpy(fw, b.fw.data(), b.fw.size() * 4);
    return FLIP_OK;
}

int flip_compute_domain_solid(int isize, int jsize, int ksize, double dx, int cfl, float *nodal, float *wu,
                              float *wv, float *ww, int *nearDims, uint8_t *nearOut) {
    if (isize <= 0 || jsize <= 0 || ksize <= 0 || !(dx > 0.0) || cfl < 1)
        return fail(FLIP_E_DOMAIN, "bad grid or CFL number");
    DomainBox b;
    b.compute(isize, jsize, ksize, dx, cfl);
    if (nodal) std::memcpy(nodal, b.nodal.data(), b.nodal.size() * 4);
    if (wu) std::memcpy(wu, b.wu.data(), b.wu.size() * 4);
    if (wv) std::memcpy(wv, b.wv.data(), b.wv.size() * 4);
    if (ww) std::memcpy(ww, b.ww.data(), b.ww.size() * 4);
    if (nearDims) { nearDims[0] = b.nsi; nearDims[1] = b.nsj; nearDims[2] = b.nsk; }
    if (nearOut) std::memcpy(nearOut, b.near.data(), b.near.size());
    return FLIP_OK;
}

int flip_set_stage_timing(flip_ctx *x, int enable) {
    if (!x) return FLIP_E_NULL;
    FLIP_SYNC_COUNT();
    CK(cudaStreamSynchronize(x->stream));
    if (enable && !x->ev[0]) {
        for (int q = 0; q <= FLIP_NUM_STAGES; q++) CK(cudaEventCreate(&x->ev[q]));
        for (int q = 0; q < 2 * (PCG_BATCH + 1); q++) CK(cudaEventCreate(&x->sweepTiming.ev[q]));
    }
    x->timing = enable != 0;
    for (int q = 0; q < FLIP_NUM_STAGES; q++) x->stageMs[q] = 0.0;
    x->timedSubsteps = 0;
    x->sweepTiming.ms = 0.0;
    x->sweepTiming.launches = 0;
    x->sweepTiming.cellSweeps = 0;
    return FLIP_OK;
}

int flip_set_sweep_orientation(flip_ctx *x, int mode) {
    if (!x) return FLIP_E_NULL;
    if (mode < -1 || mode > 1) return FLIP_E_OUT_OF_RANGE;
    x->sweepOrientation = mode;
    return FLIP_OK;
}

int flip_get_sweep_orientation(flip_ctx *x, int *last) {
    if (!x || !last) return FLIP_E_NULL;
    *last = x->pr.sl.swap;
    return FLIP_OK;
}

int flip_get_sweep_times(flip_ctx *x, double *ms, long long *launches, long long *cell_sweeps) {
    if (!x || !ms) return FLIP_E_NULL;
    *ms = x->sweepTiming.ms;
    if (launches) *launches = x->sweepTiming.launches;
    if (cell_sweeps) *cell_sweeps = x->sweepTiming.cellSweeps;
    return FLIP_OK;
}

int flip_get_stage_times(flip_ctx *x, double *ms, long long *substeps) {
    if (!x || !ms) return FLIP_E_NULL;
    for (int q = 0; q < FLIP_NUM_STAGES; q++) ms[q] = x->stageMs[q];
    if (substeps) *substeps = x->timedSubsteps;
    return FLIP_OK;
}

int flip_get_device_bytes(flip_ctx *x, long long *bytes) {
    if (!x || !bytes) return FLIP_E_NULL;
    *bytes = x->deviceBytes + x->mesh.bytes;
    return FLIP_OK;
}

// The allocations of alloc_grids and alloc_particles, summed without a device.
int flip_estimate_device_bytes(int isize, int jsize, int ksize, int particles, long long *bytes) {
    if (!bytes) return FLIP_E_NULL;
    if (isize <= 0 || jsize <= 0 || ksize <= 0 || particles < 0)
        return fail(FLIP_E_DOMAIN, "bad grid or particle count");
    const long long I = isize, J = jsize, K = ksize, nc = I * J * K;
    const long long faces = (I + 1) * J * K + I * (J + 1) * K + I * J * (K + 1);
    const long long nsl = sweep_layout_size(isize, jsize, ksize);
    const long long cap = std::max(particles, 1);
    long long b = 0;
    b += 5 * (nc + 1) * 4 + (scan_scratch_ints((int)nc) + 4) * 4 + 16;   // binning
    b += nc * 4 + (I + 1) * (J + 1) * (K + 1) * 4 + nc;                  // phi, solid phi, solid cells
    b += faces * (4 * 3 + 1 + 1);                                        // weights, velocity, saved, valid, status
    b += nc * (1 + 32 + 32 + 8 * 5 + 4 * 3 + 4) + nsl * (16 + 4 + 4);     // pressure system (s, s2, zc)
    b += (nc + 1) * 4 * 2 + nc * 4 * 2 + (scan_scratch_ints((int)nc) + 8) * 4;   // row list
    b += (PCG_MAX_PARTIALS + 32) * 8 + 64 + 16 + 32;
    b += (mic0_factor_tiles(jsize, ksize) + 1) * 4 + 64;                  // factor tiles, ticket, control
    b += sweep_exchange_words(isize, jsize, ksize) * 8 + 4096;           // sweep exchange, ranges, tables
    b += cap * (7 * 4 * 2 + 4 * 4) + (scan_scratch_ints((int)cap) + 4) * 4 + 64;   // particles
    *bytes = b;
    return FLIP_OK;
}

int flip_get_launch_count(flip_ctx *x, long long *count) {
    if (!x || !count) return FLIP_E_NULL;
    *count = x->launches;
    return FLIP_OK;
}

int flip_get_host_sync_count(flip_ctx *x, long long *count) {
    if (!x || !count) return FLIP_E_NULL;
    *count = x->hostSyncs;
    return FLIP_OK;
}

static flip_fluid_source_params default_source_params() {
    flip_fluid_source_params p{};
    p.inflow = 1;
    p.enabled = 1;
    p.substep_emissions = 1;
    p.constrained_velocity = 1;
    p.fluid_outflow = 1;
    p.outflow_inversed = 0;
    return p;
}
static int check_source_params(const flip_fluid_source_params *p) {
    for (double v : p->velocity)
        if (!std::isfinite(v)) return fail(FLIP_E_DOMAIN, "Error: fluid source velocity must be finite.");
    return FLIP_OK;
}
static flip_ctx::FluidSource *find_source(flip_ctx *x, int id) {
    for (auto &src : x->sources)
        if (src.id == id) return &src;
    return nullptr;
}
int flip_add_mesh_fluid_source(flip_ctx *x, int nverts, const float *verts, int ntris, const int *tris,
                               const flip_fluid_source_params *params, int *id) {
    if (!x || !id) return FLIP_E_NULL;
    std::vector<MeshObstacle> ms;
    int rc = obstacles_from_arrays(1, &nverts, verts, &ntris, tris, nullptr, ms);
    if (rc) return rc;
    MeshObstacle &m = ms[0];
    flip_fluid_source_params p = params ? *params : default_source_params();
    if ((rc = check_source_params(&p))) return rc;
    if (p.substep_emissions < 0) p.substep_emissions = 0;   // MeshFluidSource::setSubstepEmissions
    int constraining = 0;
    for (auto &src : x->sources) constraining += src.prm.inflow && src.prm.constrained_velocity;
    if (p.inflow && p.constrained_velocity && constraining >= MAX_CONSTRAINED_INFLOWS)
        return fail(FLIP_E_DOMAIN, "at most 8 inflow sources may constrain the fluid velocity");
    flip_ctx::FluidSource src;
    src.id = x->nextSourceId++;
    src.verts = std::move(m.verts);
    src.tris = std::move(m.tris);
    src.prm = p;
    x->sources.push_back(std::move(src));
    *id = x->sources.back().id;
    return FLIP_OK;
}
int flip_set_mesh_fluid_source_params(flip_ctx *x, int id, const flip_fluid_source_params *params) {
    if (!x || !params) return FLIP_E_NULL;
    flip_ctx::FluidSource *src = find_source(x, id);
    if (!src) return fail(FLIP_E_DOMAIN, "no mesh fluid source with this id");
    int rc = check_source_params(params);
    if (rc) return rc;
    flip_fluid_source_params p = *params;
    if (p.substep_emissions < 0) p.substep_emissions = 0;
    if (p.inflow && p.constrained_velocity && !(src->prm.inflow && src->prm.constrained_velocity)) {
        int constraining = 0;
        for (auto &o : x->sources) constraining += o.prm.inflow && o.prm.constrained_velocity;
        if (constraining >= MAX_CONSTRAINED_INFLOWS)
            return fail(FLIP_E_DOMAIN, "at most 8 inflow sources may constrain the fluid velocity");
    }
    src->prm = p;
    return FLIP_OK;
}
int flip_get_mesh_fluid_source_params(flip_ctx *x, int id, flip_fluid_source_params *params) {
    if (!x || !params) return FLIP_E_NULL;
    flip_ctx::FluidSource *src = find_source(x, id);
    if (!src) return fail(FLIP_E_DOMAIN, "no mesh fluid source with this id");
    *params = src->prm;
    return FLIP_OK;
}
int flip_remove_mesh_fluid_source(flip_ctx *x, int id) {
    if (!x) return FLIP_E_NULL;
    for (size_t q = 0; q < x->sources.size(); q++)
        if (x->sources[q].id == id) {
            FLIP_SYNC_COUNT();
            cudaStreamSynchronize(x->stream);
            x->release(x->sources[q].dphi);
            x->release(x->sources[q].dcells);
            x->release(x->sources[q].dmask);
            x->sources.erase(x->sources.begin() + q);
            x->cellBitsIds.clear();
            return FLIP_OK;
        }
    return fail(FLIP_E_DOMAIN, "no mesh fluid source with this id");
}
int flip_fluid_source_setup(int isize, int jsize, int ksize, double dx, int nverts, const float *verts, int ntris,
                            const int *tris, int *nodes, float *offset, float *phi, int *ncells, int *cells) {
    if (isize <= 0 || jsize <= 0 || ksize <= 0 || !(dx > 0.0)) return fail(FLIP_E_DOMAIN, "bad grid");
    if (!nodes || !offset || !ncells) return FLIP_E_NULL;
    std::vector<MeshObstacle> ms;
    int rc = obstacles_from_arrays(1, &nverts, verts, &ntris, tris, nullptr, ms);
    if (rc) return rc;
    const MeshObstacle &m = ms[0];
    SourceGrid g;
    fluid_source_setup(isize, jsize, ksize, dx, m.verts, m.tris, g);
    for (int a = 0; a < 3; a++) {
        nodes[a] = g.nodes[a];
        offset[a] = g.offset[a];
    }
    *ncells = (int)g.cells.size();
    if (phi) std::memcpy(phi, g.phi.data(), g.phi.size() * sizeof(float));
    if (cells) std::memcpy(cells, g.cells.data(), g.cells.size() * sizeof(int));
    return FLIP_OK;
}

int flip_set_viscosity(flip_ctx *x, double v) {
    if (!x) return FLIP_E_NULL;
    if (!(v >= 0.0)) return fail(FLIP_E_DOMAIN, "Error: viscosity must be greater than or equal to 0.");
    x->viscosityEnabled = true;
    x->viscosity = v;
    return FLIP_OK;
}
int flip_get_viscosity(flip_ctx *x, double *v) {
    if (!x || !v) return FLIP_E_NULL;
    *v = x->viscosity;
    return FLIP_OK;
}
int flip_get_viscosity_solve(flip_ctx *x, long long *rows, int *iterations, double *residual) {
    if (!x) return FLIP_E_NULL;
    if (rows) *rows = x->viscResult.rows;
    if (iterations) *iterations = x->viscResult.iterations;
    if (residual) *residual = x->viscResult.residual;
    return FLIP_OK;
}

static flip::PointForceField point_field_from(const flip_point_force_field_params &q, const float centroid[3]) {
    flip::PointForceField f;
    f.cx = centroid[0];
    f.cy = centroid[1];
    f.cz = centroid[2];
    f.strength = q.strength;
    f.falloffPower = q.falloff_power;
    f.maxForceLimitFactor = q.max_force_limit_factor;
    f.minDistanceEnabled = q.min_distance_enabled != 0;
    f.minDistance = q.min_distance;
    f.maxDistanceEnabled = q.max_distance_enabled != 0;
    f.maxDistance = q.max_distance;
    f.gravityScale = q.gravity_scale;
    f.gravityScaleWidth = q.gravity_scale_width;
    f.enabled = q.enabled != 0;
    return f;
}
int flip_enable_force_fields(flip_ctx *x, int enable) {
    if (!x) return FLIP_E_NULL;
    x->ffEnabled = enable != 0;
    return FLIP_OK;
}
int flip_is_force_fields_enabled(flip_ctx *x, int *enabled) {
    if (!x || !enabled) return FLIP_E_NULL;
    *enabled = x->ffEnabled ? 1 : 0;
    return FLIP_OK;
}
int flip_set_force_field_reduction_level(flip_ctx *x, int level) {
    if (!x) return FLIP_E_NULL;
    if (level < 1) return fail(FLIP_E_DOMAIN, "Error: reduction level must be greater than or equal to 1.");
    x->ffReduction = level;
    return FLIP_OK;
}
int flip_get_force_field_reduction_level(flip_ctx *x, int *level) {
    if (!x || !level) return FLIP_E_NULL;
    *level = x->ffReduction;
    return FLIP_OK;
}
int flip_add_point_force_field(flip_ctx *x, int nverts, const float *verts, const flip_point_force_field_params *q,
                               int *id) {
    if (!x || !q) return FLIP_E_NULL;
    // getForceFieldGrid (fluidsimulation.cpp:1640-1648) throws std::domain_error
    if (!x->ffEnabled) return fail(FLIP_E_DOMAIN, "Error: force fields must be enabled before using this method.");
    if (nverts < 0) return fail(FLIP_E_DOMAIN, "negative vertex count");
    if (nverts > 0 && !verts) return FLIP_E_NULL;
    float centroid[3];
    mesh_centroid(verts, nverts, centroid);
    flip_ctx::ForceFieldEntry e{x->nextForceFieldId++, point_field_from(*q, centroid)};
    x->forceFields.push_back(e);
    x->ffDirty = true;
    if (id) *id = e.id;
    return FLIP_OK;
}
int flip_set_point_force_field_params(flip_ctx *x, int id, const flip_point_force_field_params *q) {
    if (!x || !q) return FLIP_E_NULL;
    for (auto &e : x->forceFields)
        if (e.id == id) {
            const float centroid[3] = {e.f.cx, e.f.cy, e.f.cz};
            e.f = point_field_from(*q, centroid);
            x->ffDirty = true;
            return FLIP_OK;
        }
    return fail(FLIP_E_DOMAIN, "no force field with this id");
}
int flip_get_point_force_field_params(flip_ctx *x, int id, flip_point_force_field_params *q) {
    if (!x || !q) return FLIP_E_NULL;
    for (auto &e : x->forceFields)
        if (e.id == id) {
            const flip::PointForceField &f = e.f;
            *q = flip_point_force_field_params{f.strength, f.falloffPower, f.maxForceLimitFactor,
                                               f.minDistanceEnabled ? 1 : 0, f.minDistance,
                                               f.maxDistanceEnabled ? 1 : 0, f.maxDistance, f.gravityScale,
                                               f.gravityScaleWidth, f.enabled ? 1 : 0};
            return FLIP_OK;
        }
    return fail(FLIP_E_DOMAIN, "no force field with this id");
}
int flip_point_force_grid(int ni, int nj, int nk, double dx, int nfields, const int *nverts, const float *verts,
                          const flip_point_force_field_params *params, const float *gravity, float *u, float *v,
                          float *w) {
    if (!gravity || !u || !v || !w || (nfields > 0 && (!nverts || !params))) return FLIP_E_NULL;
    if (ni < 1 || nj < 1 || nk < 1 || !(dx > 0.0) || nfields < 0) return fail(FLIP_E_DOMAIN, "bad grid or field count");
    std::vector<flip::PointForceField> fields;
    long long off = 0;
    for (int q = 0; q < nfields; q++) {
        if (nverts[q] < 0) return fail(FLIP_E_DOMAIN, "negative vertex count");
        if (nverts[q] > 0 && !verts) return FLIP_E_NULL;
        float centroid[3];
        mesh_centroid(verts ? verts + 3 * off : nullptr, nverts[q], centroid);
        off += nverts[q];
        fields.push_back(point_field_from(params[q], centroid));
    }
    flip::ForceFieldGridHost g;
    point_force_grid(ni, nj, nk, dx, fields, gravity, g);
    std::memcpy(u, g.u.data(), g.u.size() * 4);
    std::memcpy(v, g.v.data(), g.v.size() * 4);
    std::memcpy(w, g.w.data(), g.w.size() * 4);
    return FLIP_OK;
}

int flip_set_tuning(flip_ctx *x, const flip_tuning *t) {
    if (!x || !t) return FLIP_E_NULL;
    if (t->sdf_threads != 256 && t->sdf_threads != 512 && t->sdf_threads != 1024)
        return fail(FLIP_E_DOMAIN, "sdf_threads must be 256, 512 or 1024");
    if (t->pcg_cells_per_cta < 256 || t->pcg_cells_per_cta > (1 << 20))
        return fail(FLIP_E_DOMAIN, "pcg_cells_per_cta must be in [256, 2^20]");
    if (t->sweep_orientation < -1 || t->sweep_orientation > 1)
        return fail(FLIP_E_DOMAIN, "sweep_orientation must be -1, 0 or 1");
    FLIP_SYNC_COUNT();
    cudaStreamSynchronize(x->stream);
    x->sdfThreads = t->sdf_threads;
    x->sweepOrientation = t->sweep_orientation;
    if (t->pcg_cells_per_cta != x->pcgCellsPerCta) {
        x->pcgCellsPerCta = t->pcg_cells_per_cta;
        x->pr.nPartials = pressure_partials_for(x->I, x->J, x->K, x->pcgCellsPerCta);
        for (int q = 0; q < 2; q++)   // the captured iteration batches hold the old grid
            for (int o = 0; o < 2; o++)
                if (x->pr.batchGraph[q][o]) {
                    cudaGraphExecDestroy(x->pr.batchGraph[q][o]);
                    x->pr.batchGraph[q][o] = nullptr;
                }
        for (int o = 0; o < 2; o++)
            if (x->pr.loopGraph[o]) {
                cudaGraphExecDestroy(x->pr.loopGraph[o]);
                x->pr.loopGraph[o] = nullptr;
            }
    }
    return FLIP_OK;
}
int flip_get_tuning(flip_ctx *x, flip_tuning *t) {
    if (!x || !t) return FLIP_E_NULL;
    t->sdf_threads = x->sdfThreads;
    t->pcg_cells_per_cta = x->pcgCellsPerCta;
    t->sweep_orientation = x->sweepOrientation;
    return FLIP_OK;
}

int flip_enable_surface_reconstruction(flip_ctx *x, int enable) {
    if (!x) return FLIP_E_NULL;
    x->meshEnabled = enable != 0;
    return FLIP_OK;
}
int flip_is_surface_reconstruction_enabled(flip_ctx *x, int *enabled) {
    if (!x || !enabled) return FLIP_E_NULL;
    *enabled = x->meshEnabled ? 1 : 0;
    return FLIP_OK;
}
int flip_set_surface_subdivision_level(flip_ctx *x, int n) {
    if (!x) return FLIP_E_NULL;
    if (n < 1) return fail(FLIP_E_DOMAIN, "Error: subdivision level must be greater than or equal to 1.");
    x->meshSubdivisions = n;
    return FLIP_OK;
}
int flip_get_surface_subdivision_level(flip_ctx *x, int *n) {
    if (!x || !n) return FLIP_E_NULL;
    *n = x->meshSubdivisions;
    return FLIP_OK;
}
int flip_set_surface_smoothing_value(flip_ctx *x, double s) {
    if (!x) return FLIP_E_NULL;
    x->meshSmoothValue = s;
    return FLIP_OK;
}
int flip_get_surface_smoothing_value(flip_ctx *x, double *s) {
    if (!x || !s) return FLIP_E_NULL;
    *s = x->meshSmoothValue;
    return FLIP_OK;
}
int flip_set_surface_smoothing_iterations(flip_ctx *x, int n) {
    if (!x) return FLIP_E_NULL;
    if (n < 0) return fail(FLIP_E_DOMAIN, "Error: number of smoothing iterations must be positive.");
    x->meshSmoothIterations = n;
    return FLIP_OK;
}
int flip_get_surface_smoothing_iterations(flip_ctx *x, int *n) {
    if (!x || !n) return FLIP_E_NULL;
    *n = x->meshSmoothIterations;
    return FLIP_OK;
}
int flip_set_marker_particle_scale(flip_ctx *x, double s) {
    if (!x) return FLIP_E_NULL;
    if (!(s >= 0.0)) return fail(FLIP_E_DOMAIN, "Error: marker particle scale must be greater than or equal to 0.");
    x->markerParticleScale = s;
    return FLIP_OK;
}
int flip_get_marker_particle_scale(flip_ctx *x, double *s) {
    if (!x || !s) return FLIP_E_NULL;
    *s = x->markerParticleScale;
    return FLIP_OK;
}
int flip_build_isomesh(flip_ctx *x) {
    if (!x) return FLIP_E_NULL;
    if (!x->initialized) return fail(FLIP_E_RUNTIME, "Error: FluidSimulation must be initialized before meshing.");
    LaunchTally tally(x);
    int rc = build_isomesh(x);
    if (rc) return rc;
    return sync(x);
}
int flip_get_isomesh(flip_ctx *x, int *nverts, int *ntris, float *verts, int *tris) {
    if (!x || !nverts || !ntris) return FLIP_E_NULL;
    *nverts = x->mesh.nverts;
    *ntris = x->mesh.ntris;
    if (verts && x->mesh.nverts > 0)
        CK(cudaMemcpyAsync(verts, x->mesh.verts[x->mesh.cur], 3 * sizeof(float) * (size_t)x->mesh.nverts,
                           cudaMemcpyDeviceToHost, x->stream));
    if (tris && x->mesh.ntris > 0)
        CK(cudaMemcpyAsync(tris, x->mesh.tris, 3 * sizeof(int) * (size_t)x->mesh.ntris, cudaMemcpyDeviceToHost,
                           x->stream));
    return sync(x);
}

}  // extern "C"
