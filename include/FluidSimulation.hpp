// FluidSimulation.hpp -- header-only C++ face of libflip3d_gb300.so.
//
// The same class name, constructor and method names as the reference's
// FluidSimulation (src/engine/fluidsimulation.h:117-1130) for the calls its
// driver makes on the FLIP step (src/FluidManager.cpp:9-13,47-84), so a
// caller can switch by changing the include and the namespace.  Status
// codes of the C ABI come back as the exception types the reference throws:
// std::runtime_error (update before initialize, fluidsimulation.cpp:5756),
// std::domain_error (bad arguments, :1891-1896, :5761-5765) and
// std::out_of_range (bad readback range, :2058-2063).  The reference leaves
// a failed pressure solve silent; here it is reported in
// getFrameStatsData().pressureStatus and update() does not throw for it.
// CUDA failures and bounded device waits that gave up throw flip3d::Error.
#ifndef FLIP3D_FLUIDSIMULATION_HPP
#define FLIP3D_FLUIDSIMULATION_HPP

#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "flip3d.h"

namespace flip3d {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc) {
    if (rc == FLIP_OK) return;
    std::string msg = flip_last_error();
    switch (rc) {
        case FLIP_E_RUNTIME: throw std::runtime_error(msg);
        case FLIP_E_DOMAIN: throw std::domain_error(msg);
        case FLIP_E_OUT_OF_RANGE: throw std::out_of_range(msg);
        default: throw Error(rc, msg);
    }
}

// fluidsimulation.h:102-106: size entries of 3 floats (12 bytes) each
struct FluidSimulationMarkerParticleData {
    int size = 0;
    char *positions = nullptr;
    char *velocities = nullptr;
};

// the part of FluidSimulationFrameStats (fluidsimulation.h:78-100) the FLIP step produces
struct FluidSimulationFrameStats {
    int frame = 0;
    int substeps = 0;
    double deltaTime = 0.0;
    int fluidParticles = 0;
    int pressureIterations = 0;
    double pressureError = 0.0;
    int pressureStatus = FLIP_OK;
};

// vmath::vec3 (vmath.h): three float components
struct vec3 {
    float x = 0.0f, y = 0.0f, z = 0.0f;
    vec3() = default;
    vec3(double a, double b, double c) : x((float)a), y((float)b), z((float)c) {}
};
// Triangle (triangle.h): three vertex indices
struct Triangle {
    int tri[3] = {0, 0, 0};
    Triangle() = default;
    Triangle(int a, int b, int c) : tri{a, b, c} {}
};
static_assert(sizeof(vec3) == 3 * sizeof(float) && sizeof(Triangle) == 3 * sizeof(int),
              "vertices and triangles pass to the C ABI as packed arrays");

// TriangleMesh (trianglemesh.h): the members the driver reads and writes
struct TriangleMesh {
    std::vector<vec3> vertices;
    std::vector<Triangle> triangles;
};

// A static obstacle mesh: the part of the reference's MeshObject
// (meshobject.h, meshobject.cpp:32-59, 301-309) that addMeshObstacle uses.
// The caller keeps it alive while the simulation uses it, as with the
// reference (fluidsimulation.cpp:1994-2008).
class MeshObject {
public:
    MeshObject() = default;
    MeshObject(int, int, int, double) {}
    void updateMeshStatic(const TriangleMesh &m) { mesh_ = m; }
    void setFriction(float f) {
        if (f < 0.0f || f > 1.0f) throw std::domain_error("Error: friction must be in range [0.0, 1.0].");
        friction_ = f;
    }
    float getFriction() const { return friction_; }
    const TriangleMesh &getMesh() const { return mesh_; }

private:
    TriangleMesh mesh_;
    float friction_ = 0.0f;
};

// A static mesh fluid source: the part of the reference's MeshFluidSource
// (meshfluidsource.h, meshfluidsource.cpp:30-166) the simulation reads.  The
// caller keeps it alive while it is added; its settings are read at every
// update(), as the reference reads them.
class MeshFluidSource {
public:
    MeshFluidSource() { prm_ = defaults(); }
    MeshFluidSource(int, int, int, double) { prm_ = defaults(); }
    void updateMeshStatic(const TriangleMesh &m) { mesh_ = m; }
    const TriangleMesh &getMesh() const { return mesh_; }
    void enable() { prm_.enabled = 1; }
    void disable() { prm_.enabled = 0; }
    bool isEnabled() const { return prm_.enabled != 0; }
    void setSubstepEmissions(int n) { prm_.substep_emissions = n < 0 ? 0 : n; }
    int getSubstepEmissions() const { return prm_.substep_emissions; }
    void setInflow() { prm_.inflow = 1; }
    bool isInflow() const { return prm_.inflow != 0; }
    void setOutflow() { prm_.inflow = 0; }
    bool isOutflow() const { return prm_.inflow == 0; }
    void enableFluidOutflow() { prm_.fluid_outflow = 1; }
    void disableFluidOutflow() { prm_.fluid_outflow = 0; }
    bool isFluidOutflowEnabled() const { return prm_.fluid_outflow != 0; }
    void setVelocity(vec3 v) {
        prm_.velocity[0] = v.x;
        prm_.velocity[1] = v.y;
        prm_.velocity[2] = v.z;
    }
    vec3 getVelocity() const { return vec3(prm_.velocity[0], prm_.velocity[1], prm_.velocity[2]); }
    void enableConstrainedFluidVelocity() { prm_.constrained_velocity = 1; }
    void disableConstrainedFluidVelocity() { prm_.constrained_velocity = 0; }
    bool isConstrainedFluidVelocityEnabled() const { return prm_.constrained_velocity != 0; }
    void outflowInverse() { prm_.outflow_inversed = !prm_.outflow_inversed; }
    bool isOutflowInversed() const { return prm_.outflow_inversed != 0; }
    const flip_fluid_source_params &params() const { return prm_; }

private:
    static flip_fluid_source_params defaults() {
        flip_fluid_source_params p{};
        p.inflow = 1;
        p.enabled = 1;
        p.substep_emissions = 1;
        p.constrained_velocity = 1;
        p.fluid_outflow = 1;
        return p;
    }
    TriangleMesh mesh_;
    flip_fluid_source_params prm_;
};

// ForceFieldPoint (forcefieldpoint.cpp, forcefield.cpp): a point field at the
// centroid of a static mesh's vertices.  Its parameters are pushed to the
// simulation at every update(), as the reference reads them there.
class ForceFieldPoint {
public:
    ForceFieldPoint() { prm_ = defaults(); }
    void updateMeshStatic(const TriangleMesh &m) { mesh_ = m; }
    const TriangleMesh &getMesh() const { return mesh_; }
    void enable() { prm_.enabled = 1; }
    void disable() { prm_.enabled = 0; }
    bool isEnabled() const { return prm_.enabled != 0; }
    void setStrength(float s) { prm_.strength = s; }
    float getStrength() const { return prm_.strength; }
    void setFalloffPower(float p) { prm_.falloff_power = p; }
    float getFalloffPower() const { return prm_.falloff_power; }
    void setMaxForceLimitFactor(float f) { prm_.max_force_limit_factor = f; }
    float getMaxForceLimitFactor() const { return prm_.max_force_limit_factor; }
    void enableMinDistance() { prm_.min_distance_enabled = 1; }
    void disableMinDistance() { prm_.min_distance_enabled = 0; }
    bool isMinDistanceEnabled() const { return prm_.min_distance_enabled != 0; }
    void setMinDistance(float d) { prm_.min_distance = d; }
    float getMinDistance() const { return prm_.min_distance; }
    void enableMaxDistance() { prm_.max_distance_enabled = 1; }
    void disableMaxDistance() { prm_.max_distance_enabled = 0; }
    bool isMaxDistanceEnabled() const { return prm_.max_distance_enabled != 0; }
    void setMaxDistance(float d) { prm_.max_distance = d; }
    float getMaxDistance() const { return prm_.max_distance; }
    void setGravityScale(float s) { prm_.gravity_scale = s; }
    float getGravityScale() const { return prm_.gravity_scale; }
    void setGravityScaleWidth(float w) { prm_.gravity_scale_width = w; }
    float getGravityScaleWidth() const { return prm_.gravity_scale_width; }
    const flip_point_force_field_params &params() const { return prm_; }

private:
    static flip_point_force_field_params defaults() {
        flip_point_force_field_params p{};
        p.falloff_power = 1.0f;
        p.max_force_limit_factor = 3.0f;
        p.gravity_scale = 1.0f;
        p.enabled = 1;
        return p;
    }
    TriangleMesh mesh_;
    flip_point_force_field_params prm_;
};

class FluidSimulation;
// What getForceFieldGrid() returns: addForceField registers a point field
// (the pointer is kept; the caller owns the field, as in the reference).
class ForceFieldGrid {
public:
    void addForceField(ForceFieldPoint *field);

private:
    friend class FluidSimulation;
    FluidSimulation *sim_ = nullptr;
};

class FluidSimulation {
public:
    FluidSimulation(int isize, int jsize, int ksize, double dx) : isize_(isize), jsize_(jsize), ksize_(ksize), dx_(dx) {
        check(flip_create(isize, jsize, ksize, dx, &ctx_));
    }
    ~FluidSimulation() { flip_destroy(ctx_); }
    FluidSimulation(const FluidSimulation &) = delete;
    FluidSimulation &operator=(const FluidSimulation &) = delete;

    void initialize() { check(flip_initialize(ctx_)); }
    // getGridDimensions / getCellSize / getSimulationDimensions
    // (fluidsimulation.cpp:109-133)
    void getGridDimensions(int *i, int *j, int *k) const { *i = isize_; *j = jsize_; *k = ksize_; }
    double getCellSize() const { return dx_; }
    void getSimulationDimensions(double *w, double *h, double *d) const {
        *w = (double)isize_ * dx_;
        *h = (double)jsize_ * dx_;
        *d = (double)ksize_ * dx_;
    }
    bool isInitialized() {
        int v = 0;
        check(flip_is_initialized(ctx_, &v));
        return v != 0;
    }
    void update(double dt) {
        for (auto &src : sources_) check(flip_set_mesh_fluid_source_params(ctx_, src.second, &src.first->params()));
        for (auto &f : fields_) check(flip_set_point_force_field_params(ctx_, f.second, &f.first->params()));
        int rc = flip_update(ctx_, dt);
        if (rc != FLIP_E_SOLVER_NOCONV) check(rc);
    }
    int getCurrentFrame() {
        int f = 0;
        check(flip_get_current_frame(ctx_, &f));
        return f;
    }
    void setCurrentFrame(int frame) { check(flip_set_current_frame(ctx_, frame)); }
    void addBodyForce(double fx, double fy, double fz) { check(flip_add_body_force(ctx_, fx, fy, fz)); }
    void resetBodyForce() { check(flip_reset_body_force(ctx_)); }
    void setCFLConditionNumber(int n) { check(flip_set_cfl_condition_number(ctx_, n)); }
    void setPICFLIPRatio(double r) { check(flip_set_pic_flip_ratio(ctx_, r)); }
    double getPICFLIPRatio() {
        double r = 0.0;
        check(flip_get_pic_flip_ratio(ctx_, &r));
        return r;
    }
    // enableForceFields / setForceFieldReductionLevel / getForceFieldGrid
    // (fluidsimulation.cpp:1605-1648)
    void enableForceFields() { check(flip_enable_force_fields(ctx_, 1)); }
    void disableForceFields() { check(flip_enable_force_fields(ctx_, 0)); }
    bool isForceFieldsEnabled() {
        int v = 0;
        check(flip_is_force_fields_enabled(ctx_, &v));
        return v != 0;
    }
    void setForceFieldReductionLevel(int level) { check(flip_set_force_field_reduction_level(ctx_, level)); }
    int getForceFieldReductionLevel() {
        int v = 0;
        check(flip_get_force_field_reduction_level(ctx_, &v));
        return v;
    }
    ForceFieldGrid *getForceFieldGrid() {
        if (!isForceFieldsEnabled())
            throw std::domain_error("Error: force fields must be enabled before using this method.\n");
        grid_.sim_ = this;
        return &grid_;
    }
    void addPointForceField(ForceFieldPoint *field) {
        const TriangleMesh &m = field->getMesh();
        int id = 0;
        check(flip_add_point_force_field(ctx_, (int)m.vertices.size(), reinterpret_cast<const float *>(m.vertices.data()),
                                         &field->params(), &id));
        fields_.push_back({field, id});
    }
    // setViscosity / getViscosity (fluidsimulation.cpp:1650-1670)
    void setViscosity(double v) { check(flip_set_viscosity(ctx_, v)); }
    double getViscosity() {
        double v = 0.0;
        check(flip_get_viscosity(ctx_, &v));
        return v;
    }

    // No effect: the step runs on the GPU; kept for drivers that call it.
    void setMaxThreadCount(int) {}

    // Surface reconstruction (fluidsimulation.cpp:216-300, 367-380): on by
    // default; the mesh of the last frame's first substep.
    void enableSurfaceReconstruction() { check(flip_enable_surface_reconstruction(ctx_, 1)); }
    void disableSurfaceReconstruction() { check(flip_enable_surface_reconstruction(ctx_, 0)); }
    bool isSurfaceReconstructionEnabled() {
        int v = 0;
        check(flip_is_surface_reconstruction_enabled(ctx_, &v));
        return v != 0;
    }
    void setSurfaceSubdivisionLevel(int n) { check(flip_set_surface_subdivision_level(ctx_, n)); }
    int getSurfaceSubdivisionLevel() {
        int v = 0;
        check(flip_get_surface_subdivision_level(ctx_, &v));
        return v;
    }
    void setSurfaceSmoothingValue(double s) { check(flip_set_surface_smoothing_value(ctx_, s)); }
    double getSurfaceSmoothingValue() {
        double v = 0.0;
        check(flip_get_surface_smoothing_value(ctx_, &v));
        return v;
    }
    void setSurfaceSmoothingIterations(int n) { check(flip_set_surface_smoothing_iterations(ctx_, n)); }
    int getSurfaceSmoothingIterations() {
        int v = 0;
        check(flip_get_surface_smoothing_iterations(ctx_, &v));
        return v;
    }
    void setMarkerParticleScale(double s) { check(flip_set_marker_particle_scale(ctx_, s)); }
    double getMarkerParticleScale() {
        double v = 0.0;
        check(flip_get_marker_particle_scale(ctx_, &v));
        return v;
    }
    // getIsomesh (fluidsimulation.cpp:2543-2546): copied from the device on
    // each call into the object returned.
    TriangleMesh &getIsomesh() {
        int nv = 0, nt = 0;
        check(flip_get_isomesh(ctx_, &nv, &nt, nullptr, nullptr));
        mesh_.vertices.resize((size_t)nv);
        mesh_.triangles.resize((size_t)nt);
        check(flip_get_isomesh(ctx_, &nv, &nt, reinterpret_cast<float *>(mesh_.vertices.data()),
                               reinterpret_cast<int *>(mesh_.triangles.data())));
        return mesh_;
    }

    // addMeshObstacle (fluidsimulation.cpp:1994-2008): static obstacles only.
    void addMeshObstacle(MeshObject *obstacle) {
        for (MeshObject *o : obstacles_)
            if (o == obstacle) throw std::runtime_error("Error: mesh obstacle has already been added.\n");
        const TriangleMesh &m = obstacle->getMesh();
        check(flip_add_mesh_obstacle(ctx_, (int)m.vertices.size(), reinterpret_cast<const float *>(m.vertices.data()),
                                     (int)m.triangles.size(), reinterpret_cast<const int *>(m.triangles.data()),
                                     obstacle->getFriction()));
        obstacles_.push_back(obstacle);
    }

    // addMeshFluidSource / removeMeshFluidSource / removeMeshFluidSources
    // (fluidsimulation.cpp:1953-1992): static meshes; the pointer is kept.
    void addMeshFluidSource(MeshFluidSource *source) {
        for (auto &src : sources_)
            if (src.first == source) throw std::runtime_error("Error: Mesh fluid source has already been added.\n");
        const TriangleMesh &m = source->getMesh();
        int id = 0;
        check(flip_add_mesh_fluid_source(ctx_, (int)m.vertices.size(), reinterpret_cast<const float *>(m.vertices.data()),
                                         (int)m.triangles.size(), reinterpret_cast<const int *>(m.triangles.data()),
                                         &source->params(), &id));
        sources_.push_back({source, id});
    }
    void removeMeshFluidSource(MeshFluidSource *source) {
        for (size_t q = 0; q < sources_.size(); q++)
            if (sources_[q].first == source) {
                check(flip_remove_mesh_fluid_source(ctx_, sources_[q].second));
                sources_.erase(sources_.begin() + q);
                return;
            }
        throw std::invalid_argument("Error: could not find mesh fluid source to remove.\n");
    }
    void removeMeshFluidSources() {
        for (auto &src : sources_) check(flip_remove_mesh_fluid_source(ctx_, src.second));
        sources_.clear();
    }

    // addMeshFluid (fluidsimulation.cpp:2038-2047): the mesh is copied and
    // filled with marker particles at the end of the next substep.
    void addMeshFluid(const MeshObject &fluid) { addMeshFluid(fluid, vec3(0.0, 0.0, 0.0)); }
    void addMeshFluid(const MeshObject &fluid, vec3 velocity) {
        const TriangleMesh &m = fluid.getMesh();
        check(flip_add_mesh_fluid(ctx_, (int)m.vertices.size(), reinterpret_cast<const float *>(m.vertices.data()),
                                  (int)m.triangles.size(), reinterpret_cast<const int *>(m.triangles.data()),
                                  velocity.x, velocity.y, velocity.z));
    }
    void setMarkerParticleJitterFactor(double jit) { check(flip_set_marker_particle_jitter_factor(ctx_, jit)); }
    double getMarkerParticleJitterFactor() {
        double v = 0.0;
        check(flip_get_marker_particle_jitter_factor(ctx_, &v));
        return v;
    }
    void enableJitterSurfaceMarkerParticles() { check(flip_set_jitter_surface_marker_particles(ctx_, 1)); }
    void disableJitterSurfaceMarkerParticles() { check(flip_set_jitter_surface_marker_particles(ctx_, 0)); }
    bool isJitterSurfaceMarkerParticlesEnabled() {
        int v = 0;
        check(flip_is_jitter_surface_marker_particles_enabled(ctx_, &v));
        return v != 0;
    }

    void loadMarkerParticleData(FluidSimulationMarkerParticleData data) {
        check(flip_load_marker_particle_data(ctx_, data.size, reinterpret_cast<const float *>(data.positions),
                                             reinterpret_cast<const float *>(data.velocities)));
    }
    unsigned int getNumMarkerParticles() {
        int n = 0;
        check(flip_get_num_marker_particles(ctx_, &n));
        return (unsigned int)n;
    }
    unsigned int getMarkerParticlePositionDataSize() { return 3 * sizeof(float) * getNumMarkerParticles(); }
    unsigned int getMarkerParticleVelocityDataSize() { return 3 * sizeof(float) * getNumMarkerParticles(); }
    void getMarkerParticlePositionData(char *data) {
        check(flip_get_marker_particle_position_data(ctx_, reinterpret_cast<float *>(data)));
    }
    void getMarkerParticleVelocityData(char *data) {
        check(flip_get_marker_particle_velocity_data(ctx_, reinterpret_cast<float *>(data)));
    }
    void getMarkerParticlePositionDataRange(int start, int end, char *data) {
        check(flip_get_marker_particle_position_data_range(ctx_, start, end, reinterpret_cast<float *>(data)));
    }
    void getMarkerParticleVelocityDataRange(int start, int end, char *data) {
        check(flip_get_marker_particle_velocity_data_range(ctx_, start, end, reinterpret_cast<float *>(data)));
    }
    FluidSimulationFrameStats getFrameStatsData() {
        flip_frame_stats s{};
        check(flip_get_frame_stats(ctx_, &s));
        FluidSimulationFrameStats o;
        o.frame = s.frame;
        o.substeps = s.substeps;
        o.deltaTime = s.delta_time;
        o.fluidParticles = s.fluid_particles;
        o.pressureIterations = s.pressure_iterations;
        o.pressureError = s.pressure_error;
        o.pressureStatus = s.pressure_status;
        return o;
    }

    flip_ctx *handle() { return ctx_; }

private:
    int isize_, jsize_, ksize_;
    double dx_;
    flip_ctx *ctx_ = nullptr;
    TriangleMesh mesh_;
    std::vector<MeshObject *> obstacles_;
    std::vector<std::pair<MeshFluidSource *, int>> sources_;
    std::vector<std::pair<ForceFieldPoint *, int>> fields_;
    ForceFieldGrid grid_;
};

inline void ForceFieldGrid::addForceField(ForceFieldPoint *field) { sim_->addPointForceField(field); }

}  // namespace flip3d

#endif
