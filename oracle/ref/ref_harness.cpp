// Test-only harness around the reference FLIP engine (jklae/FLIPEngine3D,
// src/engine/*).  It is compiled by oracle/build_ref.sh from the reference's
// own sources into oracle/_ref/libflipref.so and is used ONLY by the tests and
// by the golden-fixture generator to pin the C++ restatement in oracle/.
// Nothing in the product library links or loads it.
//
// This translation unit redefines private/protected as public (after the
// standard headers) so
// it can (a) set the pressure tolerance, which the reference keeps private with
// no setter (src/engine/fluidsimulation.h:1657), and (b) run one substep stage
// by stage, in the order of FluidSimulation::_stepFluid
// (src/engine/fluidsimulation.cpp:5471-5508), dumping the state between stages.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <limits>
#include <map>
#include <mutex>
#include <condition_variable>
#include <queue>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

// Standard headers above are included before the access override below.
#define private public
#define protected public
#include "fluidsimulation.h"
#include "pressuresolver.h"
#include "pcgsolver/pcgsolver.h"
#include "pcgsolver/sparsematrix.h"
#include "meshobject.h"
#include "meshfluidsource.h"
#include "forcefieldgrid.h"
#include "forcefieldpoint.h"

namespace {

struct RefSim {
    FluidSimulation *sim = nullptr;
    std::vector<MeshObject *> obstacles;   // owned here, registered with the simulation
    std::vector<MeshFluidSource *> sources;   // owned here, registered with the simulation
    std::vector<ForceField *> fields;          // owned here, registered with the force-field grid
    std::string status;
    unsigned int particleFragmentBytes = 0;   // 0: the reference's default fragments
};

template <class T>
void copyArray(Array3d<T> &a, T *out) {
    int n = a.width * a.height * a.depth;
    T *raw = a.getRawArray();
    std::memcpy(out, raw, sizeof(T) * (size_t)n);
}

void copyBool(Array3d<bool> &a, uint8_t *out) {
    int n = a.width * a.height * a.depth;
    bool *raw = a.getRawArray();
    for (int i = 0; i < n; i++) out[i] = raw[i] ? 1 : 0;
}

}  // namespace

// Buffers filled by ref_update_staged.  Any pointer may be null.
struct RefStageDump {
    float *phi;          // I*J*K   liquid SDF after post-processing
    float *u_p2g, *v_p2g, *w_p2g;           // after P2G + extrapolation
    uint8_t *vu_p2g, *vv_p2g, *vw_p2g;      // valid masks after P2G (pre-extrapolation)
    float *u_force, *v_force, *w_force;     // after body force
    float *pressure;     // I*J*K   PCG solution scattered to cells (0 elsewhere)
    double *rhs;         // I*J*K   negative divergence (0 elsewhere)
    float *u_press, *v_press, *w_press;     // after pressure apply + extrapolation
    float *u_final, *v_final, *w_final;     // after constrain
    float *u_saved, *v_saved, *w_saved;     // saved field after constrain
    float *vel_g2p;      // 3*N_before velocities after PIC/FLIP update (pre-advection)
    float *pos_adv;      // 3*N_before positions after RK3+collision (pre-removal)
    int *n_before;       // particle count at the start of the step
    int *pcg_iters;
    double *pcg_error;
};

extern "C" {

void *ref_create(int isize, int jsize, int ksize, double dx) {
    RefSim *r = new RefSim();
    r->sim = new FluidSimulation(isize, jsize, ksize, dx);
    r->sim->disableSurfaceReconstruction();
    r->sim->_logfile.disableConsole();
    return r;
}

void ref_destroy(void *h) {
    RefSim *r = (RefSim *)h;
    delete r->sim;
    for (MeshObject *o : r->obstacles) delete o;
    for (MeshFluidSource *q : r->sources) delete q;
    for (ForceField *f : r->fields) delete f;
    delete r;
}

void ref_set_threads(void *h, int n) { ((RefSim *)h)->sim->setMaxThreadCount(n); }
// The byte size of the marker-particle container's fragments
// (FragmentedVector::setFragmentByteSize, fragmentedvector.h:59-64; default
// 5e6).  Its element access computes the fragment as (int)(i * (1.0 / n))
// with n elements per fragment (fragmentedvector.h:141-153, 295-302): for
// some i that are multiples of n the product rounds below i / n and the
// access lands on the first element of the previous fragment.  Fragments
// larger than the particle count have no such index.  Set here for the
// simulation's particle container and for the load queue's, which
// loadMarkerParticleData fills and _loadMarkerParticles reads back
// (fluidsimulation.cpp:2488-2509, 2773-2786).  Only before particles are
// loaded.
void ref_set_particle_fragment_bytes(void *h, unsigned int bytes) {
    RefSim *r = (RefSim *)h;
    r->particleFragmentBytes = bytes;
    r->sim->_markerParticles.setFragmentByteSize(bytes);
}
void ref_set_pic_ratio(void *h, double ratio) { ((RefSim *)h)->sim->setPICFLIPRatio(ratio); }
void ref_add_body_force(void *h, double x, double y, double z) { ((RefSim *)h)->sim->addBodyForce(x, y, z); }
void ref_set_cfl(void *h, int c) { ((RefSim *)h)->sim->setCFLConditionNumber(c); }
void ref_set_pressure_tol(void *h, double tol) { ((RefSim *)h)->sim->_pressureSolveTolerance = tol; }
void ref_set_pressure_maxiter(void *h, int n) { ((RefSim *)h)->sim->_maxPressureSolveIterations = n; }

void ref_load_particles(void *h, int n, const float *pos, const float *vel) {
    RefSim *r = (RefSim *)h;
    if (r->particleFragmentBytes == 0) {
        FluidSimulationMarkerParticleData d;
        d.size = n;
        d.positions = (char *)pos;
        d.velocities = (char *)vel;
        r->sim->loadMarkerParticleData(d);
        return;
    }
    if (n == 0) return;
    // loadMarkerParticleData (fluidsimulation.cpp:2488-2509) with the load
    // queue's container in fragments of the chosen size
    const vmath::vec3 *positions = (const vmath::vec3 *)pos;
    const vmath::vec3 *velocities = (const vmath::vec3 *)vel;
    FluidSimulation::MarkerParticleLoadData loadData;
    loadData.particles.setFragmentByteSize(r->particleFragmentBytes);
    loadData.particles.reserve(n);
    for (int i = 0; i < n; i++) loadData.particles.push_back(MarkerParticle(positions[i], velocities[i]));
    r->sim->_markerParticleLoadQueue.push_back(loadData);
    r->sim->_isMarkerParticleLoadPending = true;
}

// The reference builds its static solid level sets (the domain box and static
// obstacles) on initialisation, with ray origins jittered by the C library's
// rand() (meshutils.cpp:95-122).  Which rays graze an edge, and so the signs
// of some nodes, depends on that jitter: the generator is reseeded to its
// start-of-process state (seed 1) first, so that a simulation set up after
// other rand() users in the same process builds the same level set as one
// set up in a fresh process.
static void seed_like_a_fresh_process(FluidSimulation *s) {
    if (!s->isInitialized()) std::srand(1);
}

void ref_initialize(void *h) {
    seed_like_a_fresh_process(((RefSim *)h)->sim);
    ((RefSim *)h)->sim->initialize();
}
void ref_update(void *h, double dt) {
    seed_like_a_fresh_process(((RefSim *)h)->sim);
    ((RefSim *)h)->sim->update(dt);
}

int ref_num_particles(void *h) { return (int)((RefSim *)h)->sim->getNumMarkerParticles(); }

void ref_get_particles(void *h, float *pos, float *vel) {
    FluidSimulation *s = ((RefSim *)h)->sim;
    if (pos) s->getMarkerParticlePositionData((char *)pos);
    if (vel) s->getMarkerParticleVelocityData((char *)vel);
}

int ref_frame_substeps(void *h) { return ((RefSim *)h)->sim->getFrameStatsData().substeps; }

void ref_get_liquid_phi(void *h, float *out) { copyArray(((RefSim *)h)->sim->_liquidSDF._phi, out); }
void ref_get_solid_phi(void *h, float *out) { copyArray(((RefSim *)h)->sim->_solidSDF._phi, out); }

void ref_get_mac(void *h, float *u, float *v, float *w) {
    MACVelocityField &m = ((RefSim *)h)->sim->_MACVelocity;
    copyArray(m._u, u);
    copyArray(m._v, v);
    copyArray(m._w, w);
}

void ref_get_weights(void *h, float *wu, float *wv, float *ww, float *wc) {
    FluidSimulation *s = ((RefSim *)h)->sim;
    s->_updateWeightGrid();
    copyArray(s->_weightGrid.U, wu);
    copyArray(s->_weightGrid.V, wv);
    copyArray(s->_weightGrid.W, ww);
    copyArray(s->_weightGrid.center, wc);
}

void ref_get_near_solid(void *h, int *dims, uint8_t *out) {
    FluidSimulation *s = ((RefSim *)h)->sim;
    dims[0] = s->_nearSolidGrid.width;
    dims[1] = s->_nearSolidGrid.height;
    dims[2] = s->_nearSolidGrid.depth;
    if (out) copyBool(s->_nearSolidGrid, out);
}

const char *ref_pressure_status(void *h) {
    RefSim *r = (RefSim *)h;
    r->status = r->sim->_pressureSolverStatus;
    return r->status.c_str();
}

// One frame of exactly one substep of length dt, run stage by stage in the
// order of FluidSimulation::update (src/engine/fluidsimulation.cpp:5755-5845)
// and _stepFluid (:5471-5508), with state dumps between the stages.  Returns
// -1 (and does nothing) if the CFL condition would split the frame.
int ref_update_staged(void *h, double dt, RefStageDump *d) {
    FluidSimulation *s = ((RefSim *)h)->sim;
    if (!s->_isSimulationInitialized) return -2;

    s->_timingData = FluidSimulation::TimingData();
    double epsdt = 1e-6;
    s->_isZeroLengthDeltaTime = dt < epsdt;
    dt = std::max(dt, epsdt);
    s->_isCurrentFrameFinished = false;
    s->_currentFrameDeltaTime = dt;
    s->_currentFrameDeltaTimeRemaining = dt;
    s->_currentFrameTimeStepNumber = 0;
    s->_isSkippedFrame = s->_isZeroLengthDeltaTime && s->_outputData.isInitialized;

    double step = fmin(s->_calculateNextTimeStep(dt), s->_currentFrameDeltaTimeRemaining);
    if (step < dt) return -1;
    s->_currentFrameTimeStep = step;
    s->_currentFrameDeltaTimeRemaining -= step;
    s->_isLastFrameTimeStep = true;

    int I = s->_isize, J = s->_jsize, K = s->_ksize;
    if (d->n_before) *d->n_before = (int)s->_markerParticles.size();

    // _stepFluid, stage by stage
    s->_launchUpdateObstacleObjectsThread(step);
    s->_joinUpdateObstacleObjectsThread();
    s->_launchUpdateLiquidLevelSetThread();
    s->_joinUpdateLiquidLevelSetThread();
    if (d->phi) copyArray(s->_liquidSDF._phi, d->phi);

    // _advectVelocityField, split so the pre-extrapolation valid mask is visible
    s->_validVelocities.reset();
    s->_MACVelocity.clear();
    if (!s->_markerParticles.empty()) {
        VelocityAdvectorParameters params;
        params.particles = &s->_markerParticles;
        params.vfield = &s->_MACVelocity;
        params.validVelocities = &s->_validVelocities;
        params.particleRadius = s->_liquidSDFParticleRadius;
        s->_velocityAdvector.advect(params);
        if (d->vu_p2g) {
            copyBool(s->_validVelocities.validU, d->vu_p2g);
            copyBool(s->_validVelocities.validV, d->vv_p2g);
            copyBool(s->_validVelocities.validW, d->vw_p2g);
        }
        s->_extrapolateFluidVelocities(s->_MACVelocity, s->_validVelocities);
    }
    if (d->u_p2g) ref_get_mac(h, d->u_p2g, d->v_p2g, d->w_p2g);

    s->_saveVelocityField();
    s->_applyBodyForcesToVelocityField(step);
    if (d->u_force) ref_get_mac(h, d->u_force, d->v_force, d->w_force);
    s->_applyViscosityToVelocityField(step);   // no-op unless setViscosity was called

    // _pressureSolve with PressureSolver::solve expanded so the solution
    // vector is visible (src/engine/pressuresolver.cpp:44-76)
    s->_updateWeightGrid();
    PressureSolverParameters params;
    params.cellwidth = s->_dx;
    params.deltaTime = step;
    params.tolerance = s->_pressureSolveTolerance;
    params.acceptableTolerance = s->_pressureSolveAcceptableTolerance;
    params.maxIterations = s->_maxPressureSolveIterations;
    params.velocityField = &s->_MACVelocity;
    params.validVelocities = &s->_validVelocities;
    params.liquidSDF = &s->_liquidSDF;
    params.solidSDF = &s->_solidSDF;
    params.weightGrid = &s->_weightGrid;
    params.isSurfaceTensionEnabled = false;

    PressureSolver ps;
    ps._initialize(params);
    ps._conditionSolidVelocityField();
    ps._initializeSurfaceTensionClusterData();
    std::vector<double> rhs(ps._matSize, 0);
    ps._calculateNegativeDivergenceVector(rhs);
    double maxAbsCoeff = 0.0;
    for (size_t i = 0; i < rhs.size(); i++) maxAbsCoeff = fmax(maxAbsCoeff, fabs(rhs[i]));
    std::vector<double> soln(ps._matSize, 0);
    int iters = 0;
    double err = 0.0;
    if (maxAbsCoeff < ps._pressureSolveTolerance) {
        ps._solverStatus = "Pressure Solver Iterations: 0\nEstimated Error: 0.0";
    } else {
        SparseMatrixd matrix(ps._matSize, 7);
        ps._calculateMatrixCoefficients(matrix);
        PCGSolver<double> solver;
        solver.setSolverParameters(ps._pressureSolveTolerance, ps._maxCGIterations);
        bool ok = solver.solve(matrix, rhs, soln, err, iters);
        bool accept = ok || (iters == ps._maxCGIterations && err < ps._pressureSolveAcceptableTolerance);
        if (accept) ps._applySolutionToVelocityField(soln);
        ps._solverStatus = accept ? "ok" : "***Pressure Solver FAILED";
    }
    s->_pressureSolverStatus = ps.getSolverStatus();
    if (d->pcg_iters) *d->pcg_iters = iters;
    if (d->pcg_error) *d->pcg_error = err;
    if (d->pressure || d->rhs) {
        if (d->pressure) std::fill(d->pressure, d->pressure + (size_t)I * J * K, 0.0f);
        if (d->rhs) std::fill(d->rhs, d->rhs + (size_t)I * J * K, 0.0);
        for (int idx = 0; idx < ps._matSize; idx++) {
            GridIndex g = ps._pressureCells[idx];
            size_t flat = (size_t)g.i + (size_t)I * ((size_t)g.j + (size_t)J * g.k);
            if (d->pressure) d->pressure[flat] = (float)soln[idx];
            if (d->rhs) d->rhs[flat] = rhs[idx];
        }
    }
    s->_extrapolateFluidVelocities(s->_MACVelocity, s->_validVelocities);
    if (d->u_press) ref_get_mac(h, d->u_press, d->v_press, d->w_press);

    s->_constrainVelocityFields();
    if (d->u_final) ref_get_mac(h, d->u_final, d->v_final, d->w_final);
    if (d->u_saved) {
        copyArray(s->_savedVelocityField._u, d->u_saved);
        copyArray(s->_savedVelocityField._v, d->v_saved);
        copyArray(s->_savedVelocityField._w, d->w_saved);
    }

    s->_updateMarkerParticleVelocities();
    if (d->vel_g2p) {
        for (size_t i = 0; i < s->_markerParticles.size(); i++) {
            vmath::vec3 v = s->_markerParticles[i].velocity;
            d->vel_g2p[3 * i + 0] = v.x;
            d->vel_g2p[3 * i + 1] = v.y;
            d->vel_g2p[3 * i + 2] = v.z;
        }
    }
    s->_deleteSavedVelocityField();

    // _advanceMarkerParticles with the pre-removal positions exposed
    {
        std::vector<vmath::vec3> positions;
        positions.reserve(s->_markerParticles.size());
        for (size_t i = 0; i < s->_markerParticles.size(); i++) positions.push_back(s->_markerParticles[i].position);
        std::vector<vmath::vec3> output(positions.size());
        int nthreads = (int)fmin(ThreadUtils::getMaxThreadCount(), positions.size());
        std::vector<int> intervals = ThreadUtils::splitRangeIntoIntervals(0, positions.size(), nthreads);
        for (int t = 0; t < nthreads; t++) {
            s->_advanceMarkerParticlesThread(step, intervals[t], intervals[t + 1], &positions, &output);
        }
        for (size_t i = 0; i < s->_markerParticles.size(); i++) {
            s->_markerParticles[i].position = output[i];
            if (d->pos_adv) {
                d->pos_adv[3 * i + 0] = output[i].x;
                d->pos_adv[3 * i + 1] = output[i].y;
                d->pos_adv[3 * i + 2] = output[i].z;
            }
        }
        s->_removeMarkerParticles(s->_currentFrameDeltaTime);
    }
    s->_updateFluidObjects();
    s->_outputSimulationData();
    s->_currentFrameTimeStepNumber++;

    s->_outputData.frameData.frame = s->_currentFrame;
    s->_outputData.frameData.substeps = s->_currentFrameTimeStepNumber;
    s->_outputData.frameData.deltaTime = dt;
    s->_outputData.frameData.fluidParticles = (int)s->_markerParticles.size();
    s->_outputData.isInitialized = true;
    s->_currentFrame++;
    s->_isCurrentFrameFinished = true;
    return 0;
}


// The reference's MIC(0) routines alone (pcgsolver.h): the factor
// factorModifiedIncompleteColesky0 on a SparseMatrixd built from a 7-point
// system over the flagged cells (rows in flat cell order; rows7 = {diag, +x,
// +y, +z} per cell, couplings mirrored into the neighbour's row), and the
// sweeps solveLower + solveLowerTransposeInPlace instantiated for float on a
// factor given per cell as {invdiag, L+x, L+y, L+z}.  Outputs per cell, 0 off
// the system; lower: the scaled column entries towards +x, +y, +z.
static void ref_unit_rows(int I, int J, int K, const uint8_t *fluid, std::vector<int> &cellOf, std::vector<int> &rowOf) {
    const size_t nc = (size_t)I * J * K;
    rowOf.assign(nc, -1);
    cellOf.clear();
    for (size_t t = 0; t < nc; t++)
        if (fluid[t]) { rowOf[t] = (int)cellOf.size(); cellOf.push_back((int)t); }
}

int ref_mic0_factor(int I, int J, int K, const uint8_t *fluid, const double *rows7, double *invdiag, double *lower) {
    std::vector<int> cellOf, rowOf;
    ref_unit_rows(I, J, K, fluid, cellOf, rowOf);
    const int n = (int)cellOf.size();
    const size_t nc = (size_t)I * J * K;
    const long long step[3] = {1, (long long)I, (long long)I * J};
    SparseMatrixd A(n);
    for (int c = 0; c < n; c++) {
        const long long t = cellOf[c];
        A.set(c, c, rows7[4 * t]);
        for (int q = 0; q < 3; q++) {
            const long long nb = t + step[q];
            if (nb < (long long)nc && fluid[nb]) {
                A.set(c, rowOf[nb], rows7[4 * t + 1 + q]);
                A.set(rowOf[nb], c, rows7[4 * t + 1 + q]);
            }
        }
    }
    SparseColumnLowerFactor<double> F;
    factorModifiedIncompleteColesky0(A, F);
    std::fill(invdiag, invdiag + nc, 0.0);
    if (lower) std::fill(lower, lower + 3 * nc, 0.0);
    for (int c = 0; c < n; c++) {
        const long long t = cellOf[c];
        invdiag[t] = F.invdiag[c];
        if (!lower) continue;
        for (unsigned int p = F.colstart[c]; p < F.colstart[c + 1]; p++) {
            const long long row = cellOf[F.rowindex[p]];
            for (int q = 0; q < 3; q++)
                if (row == t + step[q]) lower[3 * t + q] = F.value[p];
        }
    }
    return n;
}

int ref_mic0_precondition_f32(int I, int J, int K, const uint8_t *fluid, const float *factor, const float *r,
                              float *z) {
    std::vector<int> cellOf, rowOf;
    ref_unit_rows(I, J, K, fluid, cellOf, rowOf);
    const int n = (int)cellOf.size();
    const size_t nc = (size_t)I * J * K;
    const long long step[3] = {1, (long long)I, (long long)I * J};
    SparseColumnLowerFactor<float> F(n);
    for (int c = 0; c < n; c++) {
        const long long t = cellOf[c];
        F.colstart[c] = (unsigned int)F.rowindex.size();
        F.invdiag[c] = factor[4 * t];
        for (int q = 0; q < 3; q++) {
            const long long nb = t + step[q];
            if (nb < (long long)nc && fluid[nb]) {
                F.rowindex.push_back((unsigned int)rowOf[nb]);
                F.value.push_back(factor[4 * t + 1 + q]);
            }
        }
    }
    F.colstart[n] = (unsigned int)F.rowindex.size();
    std::fill(z, z + nc, 0.0f);
    if (n == 0) return 0;
    std::vector<float> rhs(n), res(n);
    for (int c = 0; c < n; c++) rhs[c] = r[cellOf[c]];
    solveLower(F, rhs, res);
    solveLowerTransposeInPlace(F, res);
    for (int c = 0; c < n; c++) z[cellOf[c]] = res[c];
    return n;
}


static TriangleMesh mesh_from_arrays(int nverts, const float *verts, int ntris, const int *tris) {
    TriangleMesh m;
    for (int v = 0; v < nverts; v++) m.vertices.push_back(vmath::vec3(verts[3 * v], verts[3 * v + 1], verts[3 * v + 2]));
    for (int t = 0; t < ntris; t++) {
        Triangle tri;
        tri.tri[0] = tris[3 * t];
        tri.tri[1] = tris[3 * t + 1];
        tri.tri[2] = tris[3 * t + 2];
        m.triangles.push_back(tri);
    }
    return m;
}

// addMeshFluid(MeshObject, vec3) with a static MeshObject built from plain
// arrays (fluidsimulation.cpp:2038-2047); the queue copies the object.
void ref_add_mesh_fluid(void *h, int nverts, const float *verts, int ntris, const int *tris, double vx, double vy,
                        double vz) {
    RefSim *r = (RefSim *)h;
    int I, J, K;
    r->sim->getGridDimensions(&I, &J, &K);
    MeshObject o(I, J, K, r->sim->getCellSize());
    o.updateMeshStatic(mesh_from_arrays(nverts, verts, ntris, tris));
    r->sim->addMeshFluid(o, vmath::vec3(vx, vy, vz));
}
void ref_set_jitter_factor(void *h, double f) { ((RefSim *)h)->sim->setMarkerParticleJitterFactor(f); }

// The seeding inputs of one fluid mesh: MeshObject::getCells
// (meshobject.cpp:101-140) as flat indices, and the mesh's level set as
// _updateAddedFluidMeshObjectQueue computes it (fluidsimulation.cpp:
// 4731-4750: MeshLevelSet over the grid, exact band 3).  rand() is reseeded
// as at the start of a process (the ray jitter draws from it).
void ref_mesh_fluid_cells(int I, int J, int K, double dx, int nverts, const float *verts, int ntris, const int *tris,
                          int *ncells, int *cells, float *phi) {
    std::srand(1);
    TriangleMesh m = mesh_from_arrays(nverts, verts, ntris, tris);
    MeshObject o(I, J, K, dx);
    o.updateMeshStatic(m);
    std::vector<GridIndex> cs;
    o.getCells(cs);
    *ncells = (int)cs.size();
    if (cells)
        for (size_t q = 0; q < cs.size(); q++) cells[q] = cs[q].i + I * (cs[q].j + J * cs[q].k);
    MeshLevelSet sdf(I, J, K, dx);
    sdf.disableVelocityData();
    TriangleMesh mm = o.getMesh();
    sdf.fastCalculateSignedDistanceField(mm, 3);
    if (phi) copyArray(sdf._phi, phi);
}

// addMeshObstacle with a static MeshObject built from plain arrays
// (fluidsimulation.cpp:1994-2008, meshobject.cpp:50-59, 301-309).
void ref_add_mesh_obstacle(void *h, int nverts, const float *verts, int ntris, const int *tris, float friction) {
    RefSim *r = (RefSim *)h;
    TriangleMesh m;
    for (int v = 0; v < nverts; v++) m.vertices.push_back(vmath::vec3(verts[3 * v], verts[3 * v + 1], verts[3 * v + 2]));
    for (int t = 0; t < ntris; t++) {
        Triangle tri;
        tri.tri[0] = tris[3 * t];
        tri.tri[1] = tris[3 * t + 1];
        tri.tri[2] = tris[3 * t + 2];
        m.triangles.push_back(tri);
    }
    int I, J, K;
    r->sim->getGridDimensions(&I, &J, &K);
    MeshObject *o = new MeshObject(I, J, K, r->sim->getCellSize());
    o->updateMeshStatic(m);
    o->setFriction(friction);
    r->obstacles.push_back(o);
    r->sim->addMeshObstacle(o);
}

// addMeshFluidSource (fluidsimulation.cpp:1953-1965) with a static
// MeshFluidSource built from plain arrays (meshfluidsource.cpp:30-49):
// inflow or outflow, velocity, substep emissions, constrained fluid velocity,
// fluid outflow and an inversed outflow as its setters make them.
void ref_add_mesh_fluid_source(void *h, int nverts, const float *verts, int ntris, const int *tris, int inflow,
                               double vx, double vy, double vz, int substep_emissions, int constrained,
                               int fluid_outflow, int inversed) {
    RefSim *r = (RefSim *)h;
    int I, J, K;
    r->sim->getGridDimensions(&I, &J, &K);
    MeshFluidSource *src = new MeshFluidSource(I, J, K, r->sim->getCellSize());
    src->updateMeshStatic(mesh_from_arrays(nverts, verts, ntris, tris));
    if (inflow) src->setInflow(); else src->setOutflow();
    src->setVelocity(vmath::vec3(vx, vy, vz));
    src->setSubstepEmissions(substep_emissions);
    if (constrained) src->enableConstrainedFluidVelocity(); else src->disableConstrainedFluidVelocity();
    if (fluid_outflow) src->enableFluidOutflow(); else src->disableFluidOutflow();
    if (inversed) src->outflowInverse();
    r->sources.push_back(src);
    r->sim->addMeshFluidSource(src);
}

// MeshFluidSource::update for a static mesh (meshfluidsource.cpp:171-214):
// the source's level set (its nodes, the position of its first node, the
// values) and MeshObject::getCells as flat indices.  rand() is reseeded as
// at the start of a process (the inside test's ray jitter draws from it).
void ref_fluid_source_setup(int I, int J, int K, double dx, int nverts, const float *verts, int ntris,
                            const int *tris, int *nodes, float *offset, float *phi, int *ncells, int *cells) {
    std::srand(1);
    MeshFluidSource src(I, J, K, dx);
    src.updateMeshStatic(mesh_from_arrays(nverts, verts, ntris, tris));
    src.update(1.0 / 60.0);
    MeshLevelSet *sdf = src.getMeshLevelSet();
    nodes[0] = sdf->_phi.width;
    nodes[1] = sdf->_phi.height;
    nodes[2] = sdf->_phi.depth;
    vmath::vec3 o = src.getMeshLevelSetOffset();
    offset[0] = o.x;
    offset[1] = o.y;
    offset[2] = o.z;
    if (phi) copyArray(sdf->_phi, phi);
    std::vector<GridIndex> cs;
    src.getCells(cs);
    *ncells = (int)cs.size();
    if (cells)
        for (size_t q = 0; q < cs.size(); q++) cells[q] = cs[q].i + I * (cs[q].j + J * cs[q].k);
}

// setViscosity (fluidsimulation.cpp:1654-1670)
void ref_set_viscosity(void *h, double v) { ((RefSim *)h)->sim->setViscosity(v); }
// the viscosity solver's status line of the last substep (empty when it did not run)
const char *ref_viscosity_status(void *h) {
    RefSim *r = (RefSim *)h;
    r->status = r->sim->_viscositySolverStatus;
    return r->status.c_str();
}

// Surface reconstruction settings (fluidsimulation.cpp:216-300, 367-376):
// enabled or not, subdivision level, smoothing value and iterations.  The
// mesher thread is joined at once (disableAsynchronousMeshing, :390-394), so
// getIsomesh() holds the mesh when update() returns.
void ref_set_surface_reconstruction(void *h, int enable, int subdivisions, double smooth_value, int smooth_iters) {
    FluidSimulation *s = ((RefSim *)h)->sim;
    if (enable) s->enableSurfaceReconstruction(); else s->disableSurfaceReconstruction();
    s->setSurfaceSubdivisionLevel(subdivisions);
    s->setSurfaceSmoothingValue(smooth_value);
    s->setSurfaceSmoothingIterations(smooth_iters);
    s->disableAsynchronousMeshing();
}

// The mesh of the simulation's current marker particles, as the first
// substep of a frame makes it (_launchOutputSurfaceMeshThread,
// fluidsimulation.cpp:5221-5239, and _outputSurfaceMeshThread, :5150-5219),
// run now on the current particles and solid level set.
void ref_mesh_now(void *h) {
    FluidSimulation *s = ((RefSim *)h)->sim;
    s->_launchOutputSurfaceMeshThread();
    if (s->_mesherThread.joinable()) s->_mesherThread.join();
}

// getIsomesh() (fluidsimulation.cpp:2543-2546): counts, and the vertices
// (xyz floats) and triangles (three ints) where the pointers are not null.
void ref_get_isomesh(void *h, int *nverts, int *ntris, float *verts, int *tris) {
    TriangleMesh &m = ((RefSim *)h)->sim->getIsomesh();
    *nverts = (int)m.vertices.size();
    *ntris = (int)m.triangles.size();
    if (verts)
        for (size_t v = 0; v < m.vertices.size(); v++) {
            verts[3 * v] = m.vertices[v].x;
            verts[3 * v + 1] = m.vertices[v].y;
            verts[3 * v + 2] = m.vertices[v].z;
        }
    if (tris)
        for (size_t t = 0; t < m.triangles.size(); t++)
            for (int q = 0; q < 3; q++) tris[3 * t + q] = m.triangles[t].tri[q];
}

// Per node of the solid level set, the friction of the closest mesh object
// (0 where none): what the constrain step averages per face
// (fluidsimulation.cpp:3785-3846).
void ref_get_node_friction(void *h, float *out) {
    FluidSimulation *s = ((RefSim *)h)->sim;
    int I, J, K;
    s->getGridDimensions(&I, &J, &K);
    for (int k = 0; k <= K; k++)
        for (int j = 0; j <= J; j++)
            for (int i = 0; i <= I; i++) {
                MeshObject *m = s->_solidSDF.getClosestMeshObject(i, j, k);
                out[i + (size_t)(I + 1) * (j + (size_t)(J + 1) * k)] = m == nullptr ? 0.0f : m->getFriction();
            }
}

// Force fields (forcefieldpoint.cpp, forcefieldgrid.cpp).  prm: strength,
// falloff power, max force limit factor, min distance enabled, min distance,
// max distance enabled, max distance, gravity scale, gravity scale width,
// enabled.
static ForceFieldPoint *point_field(int nverts, const float *verts, int ntris, const int *tris, const float *prm) {
    ForceFieldPoint *f = new ForceFieldPoint();
    f->updateMeshStatic(mesh_from_arrays(nverts, verts, ntris, tris));
    f->setStrength(prm[0]);
    f->setFalloffPower(prm[1]);
    f->setMaxForceLimitFactor(prm[2]);
    if (prm[3] != 0.0f) f->enableMinDistance(); else f->disableMinDistance();
    f->setMinDistance(prm[4]);
    if (prm[5] != 0.0f) f->enableMaxDistance(); else f->disableMaxDistance();
    f->setMaxDistance(prm[6]);
    f->setGravityScale(prm[7]);
    f->setGravityScaleWidth(prm[8]);
    if (prm[9] != 0.0f) f->enable(); else f->disable();
    return f;
}

void ref_enable_force_fields(void *h, int reduction) {
    RefSim *r = (RefSim *)h;
    r->sim->enableForceFields();
    r->sim->setForceFieldReductionLevel(reduction);
}

void ref_add_point_force_field(void *h, int nverts, const float *verts, int ntris, const int *tris, const float *prm) {
    RefSim *r = (RefSim *)h;
    ForceFieldPoint *f = point_field(nverts, verts, ntris, tris, prm);
    r->fields.push_back(f);
    r->sim->getForceFieldGrid()->addForceField(f);
}

// ForceFieldGrid::update of a fresh grid: fields q = 0..nfields-1 with
// nverts[q] / ntris[q] consecutive vertices / triangles (indices local to the
// field) and 10 parameters each; the grid's u, v, w faces.
void ref_point_force_grid(int ni, int nj, int nk, double dx, int nfields, const int *nverts, const float *verts,
                          const int *ntris, const int *tris, const float *prms, const float *gravity, float *u,
                          float *v, float *w) {
    ForceFieldGrid grid;
    grid.initialize(ni, nj, nk, dx);
    std::vector<ForceFieldPoint *> fields;
    size_t vo = 0, to = 0;
    for (int q = 0; q < nfields; q++) {
        fields.push_back(point_field(nverts[q], verts + 3 * vo, ntris[q], tris + 3 * to, prms + 10 * q));
        grid.addForceField(fields.back());
        vo += nverts[q];
        to += ntris[q];
    }
    grid.setGravityVector(vmath::vec3(gravity[0], gravity[1], gravity[2]));
    grid.update(0.0, 0.0);
    copyArray(grid._forceField._u, u);
    copyArray(grid._forceField._v, v);
    copyArray(grid._forceField._w, w);
    for (ForceFieldPoint *f : fields) delete f;
}

}  // extern "C"
