/*
 * flip3d.h -- C ABI of the GB300 FLIP step (libflip3d_gb300.so).
 *
 * Drop-in for the hot path of jklae/FLIPEngine3D's C++ class FluidSimulation
 * (src/engine/fluidsimulation.h:117-1130; the FLIP Fluids engine 1.0.9b):
 * construct, add body forces, set the PIC/FLIP ratio, load marker particles,
 * initialize, update(dt), read particles back.  Plain pointers and sizes
 * only.  Every call returns a status code; the header-only C++ shim in
 * include/FluidSimulation.hpp turns them back into the reference's
 * exception types.
 *
 * Threading: a context is not re-entrant; calls on one context must not
 * overlap.  All device work of a context is ordered on one CUDA stream
 * (its own, or the one given by flip_set_stream).
 */
#ifndef FLIP3D_H
#define FLIP3D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The first three mirror the exception classes the reference
 * throws (fluidsimulation.cpp: runtime_error 5756-5759, domain_error
 * 1891-1896/5761-5765, out_of_range 2058-2063). */
#define FLIP_OK 0
#define FLIP_E_RUNTIME (-1)        /* e.g. update() before initialize()          */
#define FLIP_E_DOMAIN (-2)         /* argument out of its domain                 */
#define FLIP_E_OUT_OF_RANGE (-3)   /* bad particle index range                   */
#define FLIP_E_SOLVER_NOCONV (-4)  /* pressure solve failed (reported, not fatal) */
#define FLIP_E_DEVICE_TIMEOUT (-5) /* a bounded device wait gave up              */
#define FLIP_E_CUDA (-6)           /* CUDA runtime error (no device, launch...)  */
#define FLIP_E_NOMEM (-7)          /* device allocation failed                   */
#define FLIP_E_NULL (-8)           /* null context or pointer                    */

typedef struct flip_ctx flip_ctx;

/* Frame statistics, the part of FluidSimulationFrameStats
 * (fluidsimulation.h:78-100) the hot path produces. */
typedef struct flip_frame_stats {
    int frame;
    int substeps;
    double delta_time;
    int fluid_particles;
    int pressure_iterations;  /* of the last substep */
    double pressure_error;    /* |r|inf of the last substep */
    int pressure_status;      /* FLIP_OK or FLIP_E_SOLVER_NOCONV */
    int pressure_cells;       /* rows of the last substep's pressure system */
} flip_frame_stats;

/* Stages of one substep, for flip_get_stage_times. */
#define FLIP_STAGE_LIQUID_SDF 0   /* liquid level set + solid post-process      */
#define FLIP_STAGE_P2G 1          /* P2G splat + velocity extrapolation        */
#define FLIP_STAGE_FORCE 2        /* save field + body force                   */
#define FLIP_STAGE_PRESSURE 3     /* system build, MIC(0), PCG, pressure apply */
#define FLIP_STAGE_CONSTRAIN 4    /* extrapolation + constrain                 */
#define FLIP_STAGE_ADVECT 5       /* PIC/FLIP, RK3, collision, removal tests   */
#define FLIP_STAGE_BINNING 6      /* counting sort by cell + removal           */
#define FLIP_NUM_STAGES 7

/* Stage dump of one single-substep frame (test and debug interface); any
 * pointer may be NULL.  Face grids are (I+1)*J*K, I*(J+1)*K, I*J*(K+1); cell
 * grids I*J*K; flat index i + ni*(j + nj*k).  Particle arrays are 3*n floats
 * in the reference's particle order. */
typedef struct flip_stage_dump {
    float *phi;
    float *u_p2g, *v_p2g, *w_p2g;
    uint8_t *vu_p2g, *vv_p2g, *vw_p2g;
    float *u_force, *v_force, *w_force;
    float *pressure;
    double *rhs;
    float *u_press, *v_press, *w_press;
    float *u_final, *v_final, *w_final;
    float *u_saved, *v_saved, *w_saved;
    float *vel_g2p;
    float *pos_adv;
    int *n_before;
    int *pcg_iters;
    double *pcg_error;
} flip_stage_dump;

/* FluidSimulation(int isize, int jsize, int ksize, double dx)
 * (fluidsimulation.h:127, fluidsimulation.cpp:49-52).  Binds the current
 * CUDA device.  FLIP_E_DOMAIN for non-positive sizes. */
int flip_create(int isize, int jsize, int ksize, double dx, flip_ctx **out);
int flip_destroy(flip_ctx *ctx);

/* Order the context's device work on an existing cudaStream_t (NULL: the
 * context's own stream). */
int flip_set_stream(flip_ctx *ctx, void *cuda_stream);

/* setPICFLIPRatio (fluidsimulation.cpp:1891-1903): r in [0,1] is the PIC
 * fraction; FLIP blend 0.95 is r = 0.05 (the default). */
int flip_set_pic_flip_ratio(flip_ctx *ctx, double ratio);
int flip_get_pic_flip_ratio(flip_ctx *ctx, double *ratio);

/* addBodyForce(double fx, double fy, double fz) (fluidsimulation.cpp:1582-1590) */
int flip_add_body_force(flip_ctx *ctx, double fx, double fy, double fz);
/* resetBodyForce (fluidsimulation.cpp:1598-1603) */
int flip_reset_body_force(flip_ctx *ctx);

/* setCFLConditionNumber (fluidsimulation.h:844) */
int flip_set_cfl_condition_number(flip_ctx *ctx, int n);

/* Pressure-solve controls.  The reference keeps these private
 * (fluidsimulation.h:1657-1659: tolerance 1e-9, acceptable 1.0, 1000
 * iterations); they are exposed here so the workload's tolerance can be set. */
int flip_set_pressure_tolerance(flip_ctx *ctx, double tol);
int flip_set_max_pressure_iterations(flip_ctx *ctx, int n);

/* loadMarkerParticleData(FluidSimulationMarkerParticleData)
 * (fluidsimulation.cpp:2488-2509): n packed xyz float triples each, copied
 * on the call, applied at flip_initialize (particles outside the domain box
 * are dropped, fluidsimulation.cpp:2773-2786). */
int flip_load_marker_particle_data(flip_ctx *ctx, int n, const float *positions, const float *velocities);
/* Same, from device memory (no host copy). */
int flip_load_marker_particle_data_device(flip_ctx *ctx, int n, const float *d_positions,
                                          const float *d_velocities);

/* initialize() (fluidsimulation.cpp:82-88) */
int flip_initialize(flip_ctx *ctx);
int flip_is_initialized(flip_ctx *ctx, int *yes);

/* update(double dt) (fluidsimulation.cpp:5755-5845): one frame, split into
 * 1..6 CFL substeps.  FLIP_E_RUNTIME before initialize, FLIP_E_DOMAIN for
 * dt < 0.  A failed pressure solve is reported through the frame stats, as
 * the reference only records it in its status string. */
int flip_update(flip_ctx *ctx, double dt);
/* As flip_update for a frame that is exactly one substep, filling the stage
 * dump (FLIP_E_RUNTIME if the CFL condition would split the frame). */
int flip_update_staged(flip_ctx *ctx, double dt, flip_stage_dump *dump);

/* getNumMarkerParticles (fluidsimulation.cpp:2050-2052) */
int flip_get_num_marker_particles(flip_ctx *ctx, int *n);
/* getMarkerParticlePositionData / VelocityData (fluidsimulation.cpp:2408-2420):
 * 3*n floats in the reference's particle order. */
int flip_get_marker_particle_position_data(flip_ctx *ctx, float *out);
int flip_get_marker_particle_velocity_data(flip_ctx *ctx, float *out);
/* ...DataRange (fluidsimulation.cpp:2314-2336): FLIP_E_DOMAIN on a bad range. */
int flip_get_marker_particle_position_data_range(flip_ctx *ctx, int start, int end, float *out);
int flip_get_marker_particle_velocity_data_range(flip_ctx *ctx, int start, int end, float *out);
/* Device-side readback (cell order, not the reference's order): positions
 * and velocities as 3 planes of n floats each. */
int flip_get_marker_particle_data_device(flip_ctx *ctx, float *d_positions, float *d_velocities);

/* getFrameStatsData (fluidsimulation.cpp:2302-2304), getCurrentFrame (:94-96) */
int flip_get_frame_stats(flip_ctx *ctx, flip_frame_stats *out);
int flip_get_current_frame(flip_ctx *ctx, int *frame);
/* setCurrentFrame (fluidsimulation.cpp:98-103): the frame number the next
 * update() runs as.  With marker particles loaded from a saved state, a
 * frame number above 0 makes the first substep's CFL speed the particles'
 * own (fluidsimulation.cpp:5593-5599), so the run resumes as it left off.
 * FLIP_E_DOMAIN for a negative frame. */
int flip_set_current_frame(flip_ctx *ctx, int frame);

/* Grid state readback for tests (sizes as in flip_stage_dump). */
int flip_get_liquid_sdf(flip_ctx *ctx, float *phi);
int flip_get_solid_sdf(flip_ctx *ctx, float *nodal_phi);   /* (I+1)*(J+1)*(K+1) */
int flip_get_mac_velocity(flip_ctx *ctx, float *u, float *v, float *w);
int flip_get_face_weights(flip_ctx *ctx, float *wu, float *wv, float *ww);

/* addMeshObstacle(MeshObject *) (fluidsimulation.cpp:1994-2008) for a static
 * obstacle: a triangle mesh of nverts vertices (xyz floats, world space) and
 * ntris triangles (three vertex indices each), and the friction of its
 * surface (MeshObject::setFriction, meshobject.cpp:301-309; in [0, 1]),
 * copied on the call.  The solid level set, face weights and near-solid grid
 * are rebuilt before the next step: the obstacle's level set over the
 * sub-grid its bounding box spans, unioned with the domain walls'
 * (fluidsimulation.cpp:2927-2966).  Animated and inverted obstacles are not
 * supported.  FLIP_E_DOMAIN for a bad index, count, vertex or friction. */
int flip_add_mesh_obstacle(flip_ctx *ctx, int nverts, const float *verts, int ntris, const int *tris,
                           float friction);

/* addMeshFluid(MeshObject, vec3 velocity) (fluidsimulation.cpp:2038-2047):
 * queue a static triangle mesh (arrays as flip_add_mesh_obstacle) to be
 * filled with marker particles moving at (vx, vy, vz), copied on the call.
 * The queue is filled at the end of the next substep
 * (_updateAddedFluidMeshObjectQueue, :4724-4759): every cell around a grid
 * node inside the mesh gets a particle at the centre of each of its eight
 * sub-cells where the mesh's level set is <= 0 and the solid level set is
 * positive, unless a particle already holds that sub-cell; particles deeper
 * than one cell (all of them with surface jitter on) are jittered by up to
 * 0.25 (jitter factor - 0.001) dx per axis.  On frame 0 the first substep's
 * length uses the queued meshes' speeds (_predictMaximumMarkerParticleSpeed,
 * :5529-5550).  The reference draws the jitter from rand(); here it is a
 * counter-based hash, so runs repeat; at jitter factor 0.001 it is zero and
 * the particles are the reference's.  FLIP_E_DOMAIN for a bad index, count,
 * vertex or velocity. */
int flip_add_mesh_fluid(flip_ctx *ctx, int nverts, const float *verts, int ntris, const int *tris, double vx,
                        double vy, double vz);
/* setMarkerParticleJitterFactor / getMarkerParticleJitterFactor
 * (fluidsimulation.cpp:180-195; >= 0, default 0) and
 * enable/disableJitterSurfaceMarkerParticles (:197-210; default off). */
int flip_set_marker_particle_jitter_factor(flip_ctx *ctx, double jitter);
int flip_get_marker_particle_jitter_factor(flip_ctx *ctx, double *jitter);
int flip_set_jitter_surface_marker_particles(flip_ctx *ctx, int enable);
int flip_is_jitter_surface_marker_particles_enabled(flip_ctx *ctx, int *enabled);

/* The seeding inputs of one fluid mesh, without a device: the cells around
 * the grid nodes inside the mesh (MeshObject::getCells, meshobject.cpp:
 * 101-140), ascending flat index i + I (j + J k), and the mesh's level set on
 * the (I+1)*(J+1)*(K+1) nodes (exact within 3 cells, negative inside;
 * MeshLevelSet::fastCalculateSignedDistanceField, meshlevelset.cpp:572-601).
 * cells holds up to I*J*K entries; cells and phi may be NULL. */
int flip_mesh_fluid_cells(int isize, int jsize, int ksize, double dx, int nverts, const float *verts, int ntris,
                          const int *tris, int *ncells, int *cells, float *phi);

/* The solid set-up of the first step with static mesh obstacles, without a
 * device: nodal solid level set, fluid face weights, near-solid grid (as in
 * flip_compute_domain_solid) and the face friction of the constrain step
 * (fu/fv/fw, face grids; fluidsimulation.cpp:3785-3846).  Obstacle q has
 * nverts[q] vertices, consecutive in verts, and ntris[q] triangles with
 * indices local to it, consecutive in tris; friction may be NULL (none).
 * Any output may be NULL. */
int flip_compute_solid(int isize, int jsize, int ksize, double dx, int cfl, int nobstacles, const int *nverts,
                       const float *verts, const int *ntris, const int *tris, const float *friction,
                       float *nodal_phi, float *wu, float *wv, float *ww, int *near_dims, uint8_t *near,
                       float *fu, float *fv, float *fw);

/* Static wall set-up of initialize()/the first step, without a device: the
 * domain-box solid level set on the (I+1)*(J+1)*(K+1) nodes, the fluid face
 * weights and the coarse near-solid grid (dims written to near_dims[3];
 * `near` may be NULL to query them).  Restates _updateSolidLevelSet /
 * _updateWeightGrid / _updateNearSolidGrid for the domain walls
 * (fluidsimulation.cpp:3028-3126, 3690-3730). */
int flip_compute_domain_solid(int isize, int jsize, int ksize, double dx, int cfl, float *nodal_phi, float *wu,
                              float *wv, float *ww, int *near_dims, uint8_t *near);

/* Per-stage device time: CUDA events recorded on the context's stream at the
 * stage boundaries of every substep, summed.  flip_set_stage_timing enables
 * or disables the events and resets the sums; flip_get_stage_times writes
 * FLIP_NUM_STAGES milliseconds and the number of substeps summed. */
int flip_set_stage_timing(flip_ctx *ctx, int enable);
int flip_get_stage_times(flip_ctx *ctx, double *ms, long long *substeps);
/* While stage timing is on: device time of the MIC(0) preconditioner sweeps
 * (the kernels of solveLower / solveLowerTransposeInPlace, pcgsolver.h:192-221),
 * summed; the number of sweep kernels timed; and the sum over them of the
 * pressure rows each swept. */
int flip_get_sweep_times(flip_ctx *ctx, double *ms, long long *launches, long long *cell_sweeps);

/* Orientation of the preconditioner sweep tiles: -1 (the default) picks it
 * per solve from the extent of the pressure rows, 0 runs the tile lanes along
 * j, 1 along k.  Results do not depend on it: both keep the reference's
 * order of operations.  flip_get_sweep_orientation reports the orientation
 * of the last solve.  No counterpart in the reference. */
int flip_set_sweep_orientation(flip_ctx *ctx, int mode);
int flip_get_sweep_orientation(flip_ctx *ctx, int *last);

/* The particles as binned on the device (test and debug interface): after
 * initialize() and every update(), the particles are stored sorted by cell
 * (flat index of floor(p / dx)) and, within a cell, by id, the rank in load
 * order that the reference keeps through removals.  pos: 3 planes of n
 * floats (x..., y..., z...); ids: n values; cell_start: I*J*K + 1 offsets
 * of each cell's run.  Any pointer may be NULL. */
int flip_get_binned_particles(flip_ctx *ctx, float *pos, unsigned int *ids, int *cell_start);

/* Fault injection for the bounded device waits (test interface).  Every
 * wait of the factor's and the sweeps' wavefronts gives up after `polls`
 * poll rounds (0 restores the default, about a second) and the update
 * returns FLIP_E_DEVICE_TIMEOUT; the context stays usable.  With the stall
 * on, the sweeps' tiles await edge terms under an epoch no tile publishes,
 * so any tile with an upstream neighbour tile waits until its limit runs
 * out.  Nothing faults or hangs: each wait ends at its limit. */
int flip_set_device_wait_limit(flip_ctx *ctx, unsigned int polls);
int flip_inject_sweep_stall(flip_ctx *ctx, int on);

/* The pressure solve's MIC(0) preconditioner alone, on a 7-point system the
 * caller gives (unit interface; host arrays in flat cell order, device
 * buffers allocated per call).  The system's rows are the cells flagged in
 * `fluid`, which must lie strictly inside the I x J x K grid; rows holds
 * {diag, to +x, to +y, to +z} per cell as doubles, zero towards unflagged
 * neighbours.
 *   flip_mic0_factor: the inverse pivots of factorModifiedIncompleteColesky0
 *     (pcgsolver.h:70-185, tau 0.97, pivot floor 0.25) into invdiag (one
 *     double per cell, 0 off the system), by the solve's wavefront kernels.
 *   flip_mic0_precondition: z = M^-1 r by the solve's FP32 wavefront sweeps,
 *     solveLower then solveLowerTransposeInPlace (pcgsolver.h:192-221), with
 *     the factor given as {invdiag, L to +x, L to +y, L to +z} floats per cell;
 *     orientation 0 or 1 picks the sweep tiles' lane axis (j or k).
 * FLIP_E_DOMAIN for a flagged cell on the border, FLIP_E_DEVICE_TIMEOUT if a
 * bounded wait gave up. */
int flip_mic0_factor(int isize, int jsize, int ksize, const uint8_t *fluid, const double *rows, double *invdiag);
int flip_mic0_precondition(int isize, int jsize, int ksize, const uint8_t *fluid, const float *factor,
                           const float *r, float *z, int orientation);

/* Number of this library's kernel launches issued so far on the context. */
int flip_get_launch_count(flip_ctx *ctx, long long *count);

/* Number of times this library's calls on the context waited on the device
 * (stream or event synchronisations) so far. */
int flip_get_host_sync_count(flip_ctx *ctx, long long *count);

/* setViscosity / getViscosity (fluidsimulation.cpp:1650-1670): a constant
 * viscosity >= 0 (FLIP_E_DOMAIN otherwise) turns the viscosity step on;
 * each substep then constrains the field and solves Batty's variational
 * viscosity system after the body force (_applyViscosityToVelocityField,
 * :3592-3640).  The system's set-up (face states, liquid volume fractions,
 * rows) is the reference's; it is solved by Jacobi-preconditioned CG in
 * FP64 to a relative residual of 1e-9, where the reference runs an FP32
 * MIC(0)-PCG to 1e-4, so velocities agree to the reference's own solver
 * tolerance.  flip_get_viscosity_solve reports the last substep's system
 * size, iterations and relative residual (rows 0: the solve did not run). */
int flip_set_viscosity(flip_ctx *ctx, double viscosity);
int flip_get_viscosity(flip_ctx *ctx, double *viscosity);
int flip_get_viscosity_solve(flip_ctx *ctx, long long *rows, int *iterations, double *residual);

/* Force fields (enableForceFields, setForceFieldReductionLevel,
 * getForceFieldGrid()->addForceField; fluidsimulation.cpp:1605-1647,
 * forcefieldgrid.cpp, forcefieldpoint.cpp): point fields at the centroid of a
 * static mesh.  With force fields on, the body-force step adds the force-field
 * grid instead of the constant body force (_applyBodyForcesToVelocityField,
 * :3566-3583): every field's strength / r^falloff along the direction from the
 * point (capped at max_force_limit_factor * |strength|; faces nearer than the
 * minimum distance take it, faces beyond the maximum distance none), plus the
 * body force scaled near each field by gravity_scale over gravity_scale_width,
 * on a grid of ceil(I / level) x ... cells of size level * dx, interpolated at
 * the faces (gravity outside it).  The grid is rebuilt at the first substep of
 * a frame after a field or the body force changed (_updateForceFieldGrid,
 * :3440-3448).  Fields are added once force fields are on (FLIP_E_DOMAIN
 * otherwise, as getForceFieldGrid throws std::domain_error); the reduction level (>= 1,
 * FLIP_E_DOMAIN otherwise) is taken when the grid is first built.  The
 * reference's getForceFieldReductionLevel returns the current frame
 * (fluidsimulation.cpp:1623-1625); flip_get_force_field_reduction_level
 * returns the level. */
typedef struct {
    float strength;               /* ForceField defaults: 0 */
    float falloff_power;          /* 1 */
    float max_force_limit_factor; /* 3 */
    int min_distance_enabled;     /* 0 */
    float min_distance;           /* 0 */
    int max_distance_enabled;     /* 0 */
    float max_distance;           /* 0 */
    float gravity_scale;          /* 1 */
    float gravity_scale_width;    /* 0 */
    int enabled;                  /* 1 */
} flip_point_force_field_params;
int flip_enable_force_fields(flip_ctx *ctx, int enable);
int flip_is_force_fields_enabled(flip_ctx *ctx, int *enabled);
int flip_set_force_field_reduction_level(flip_ctx *ctx, int level);
int flip_get_force_field_reduction_level(flip_ctx *ctx, int *level);
int flip_add_point_force_field(flip_ctx *ctx, int nverts, const float *verts,
                               const flip_point_force_field_params *params, int *id);
int flip_set_point_force_field_params(flip_ctx *ctx, int id, const flip_point_force_field_params *params);
int flip_get_point_force_field_params(flip_ctx *ctx, int id, flip_point_force_field_params *params);
/* The force-field grid without a device (ForceFieldGrid::update from a
 * cleared grid): nfields point fields, field q's nverts[q] vertices
 * consecutive in verts, under the body force gravity[3], on an ni x nj x nk
 * grid of cell size dx; u, v, w receive (ni+1) nj nk, ni (nj+1) nk and
 * ni nj (nk+1) floats, flat i fastest. */
int flip_point_force_grid(int ni, int nj, int nk, double dx, int nfields, const int *nverts, const float *verts,
                          const flip_point_force_field_params *params, const float *gravity, float *u, float *v,
                          float *w);

/* Tuning knobs of the device kernels, no counterpart in the reference: the
 * liquid-SDF CTA size (256, 512 or 1024 threads), the grid cells per CTA of
 * the PCG row kernels' reduction grid (256 .. 2^20), and the preconditioner
 * sweep orientation (as flip_set_sweep_orientation).  A different reduction
 * grid sums the PCG's dot products in another order, so results move in the
 * last bits; the others leave them as they are.  Defaults 512, 4096, -1.
 * flipengine3d_gb300/autotune.py measures them per grid size and writes the
 * table the Python face applies. */
typedef struct flip_tuning {
    int sdf_threads;
    int pcg_cells_per_cta;
    int sweep_orientation;
} flip_tuning;
int flip_set_tuning(flip_ctx *ctx, const flip_tuning *tuning);
int flip_get_tuning(flip_ctx *ctx, flip_tuning *tuning);

/* Mesh fluid sources: addMeshFluidSource / removeMeshFluidSource
 * (fluidsimulation.cpp:1953-1992) with a static MeshFluidSource
 * (meshfluidsource.h).  The mesh (arrays as flip_add_mesh_obstacle) is
 * copied; `params` NULL gives the reference's defaults (meshfluidsource.h:
 * 111-124): an enabled inflow emitting once per substep at velocity 0 and
 * constraining the fluid velocity, fluid outflow on, not inversed.  Per
 * substep, as the reference:
 *   - an enabled inflow that constrains the fluid velocity keeps the body
 *     force off the faces where its level set is negative, and gives its
 *     velocity to the particles in its cells where the level set is not
 *     positive (:3372-3440, 4109-4170; like the reference, these two read
 *     the level set at the world position without the level set's offset);
 *   - an enabled inflow emits particles into its cells as addMeshFluid does,
 *     `substep_emissions` times per substep, or only at a frame's first
 *     substep when 0 (:4564-4606, 4676-4698);
 *   - an enabled outflow with fluid outflow on removes the particles in its
 *     cells where its level set is negative, or with outflow_inversed those
 *     outside its cells or where the level set is not negative (:4608-4674);
 *   - frame 0's first substep length counts the enabled inflows' speeds
 *     (:5529-5551).
 * The source's level set covers the cells its bounding box spans, padded by 4
 * cells, exact in a band of 2 (meshfluidsource.cpp:171-214, 300-318).  Animated
 * sources, appended object velocity and diffuse outflow are not restated.
 * `id` identifies the source in the other calls; at most 8 inflows may
 * constrain the fluid velocity at once (FLIP_E_DOMAIN). */
typedef struct flip_fluid_source_params {
    int inflow;                 /* 1 inflow, 0 outflow (setInflow / setOutflow)          */
    int enabled;                /* enable / disable                                      */
    int substep_emissions;      /* setSubstepEmissions: negative counts as 0             */
    int constrained_velocity;   /* enable/disableConstrainedFluidVelocity                */
    int fluid_outflow;          /* enable/disableFluidOutflow                            */
    int outflow_inversed;       /* outflowInverse toggles it                              */
    double velocity[3];         /* setVelocity                                           */
} flip_fluid_source_params;
int flip_add_mesh_fluid_source(flip_ctx *ctx, int nverts, const float *verts, int ntris, const int *tris,
                               const flip_fluid_source_params *params, int *id);
int flip_set_mesh_fluid_source_params(flip_ctx *ctx, int id, const flip_fluid_source_params *params);
int flip_get_mesh_fluid_source_params(flip_ctx *ctx, int id, flip_fluid_source_params *params);
int flip_remove_mesh_fluid_source(flip_ctx *ctx, int id);
/* A source's set-up without a device: the nodes and first-node position of
 * its level set, the level set (nodes[0]*nodes[1]*nodes[2] floats, flat i
 * fastest), and its cells (ascending flat indices, up to I*J*K).  phi and
 * cells may be NULL. */
int flip_fluid_source_setup(int isize, int jsize, int ksize, double dx, int nverts, const float *verts, int ntris,
                            const int *tris, int *nodes, float *offset, float *phi, int *ncells, int *cells);

/* Surface reconstruction, the mesh getIsomesh() returns (fluidsimulation.cpp:
 * 2543-2546).  As in the reference, it is on by default and runs after the
 * first substep of every frame (_outputSimulationData, :5444-5464): the
 * marker particles' surface by marching cubes on the grid subdivided
 * `subdivision level` times, then smoothed (_outputSurfaceMeshThread,
 * :5150-5219; ParticleMesher, Polygonizer3d, TriangleMesh::smooth).  Vertices
 * and triangles are those the reference makes from the same particles.  Not
 * restated: polygonizer slices other than 1, the preview mesh, meshing
 * volumes, surface motion blur, inverted contact normals and removal near
 * the domain (all off by default in the reference); the domain offset and
 * scale are the identity.
 *   enable/disable/isSurfaceReconstructionEnabled (:367-380);
 *   set/getSurfaceSubdivisionLevel (:216-231; FLIP_E_DOMAIN below 1);
 *   set/getSurfaceSmoothingValue (:250-259) and ...Iterations (:261-276;
 *   FLIP_E_DOMAIN below 0); set/getMarkerParticleScale (:163-179; the mesher's
 *   particle radius is the marker particle radius times this, default 3;
 *   FLIP_E_DOMAIN below 0).
 * flip_build_isomesh meshes the current particles now, as the first substep
 * of a frame would (FLIP_E_RUNTIME before initialize).  flip_get_isomesh
 * writes the counts and, where the pointers are not NULL, the vertices (3
 * floats each) and triangles (3 vertex indices each). */
int flip_enable_surface_reconstruction(flip_ctx *ctx, int enable);
int flip_is_surface_reconstruction_enabled(flip_ctx *ctx, int *enabled);
int flip_set_surface_subdivision_level(flip_ctx *ctx, int n);
int flip_get_surface_subdivision_level(flip_ctx *ctx, int *n);
int flip_set_surface_smoothing_value(flip_ctx *ctx, double value);
int flip_get_surface_smoothing_value(flip_ctx *ctx, double *value);
int flip_set_surface_smoothing_iterations(flip_ctx *ctx, int n);
int flip_get_surface_smoothing_iterations(flip_ctx *ctx, int *n);
int flip_set_marker_particle_scale(flip_ctx *ctx, double scale);
int flip_get_marker_particle_scale(flip_ctx *ctx, double *scale);
int flip_build_isomesh(flip_ctx *ctx);
int flip_get_isomesh(flip_ctx *ctx, int *nverts, int *ntris, float *verts, int *tris);

/* Device memory of a context (flip_get_device_bytes), and the same figure
 * for a scene not yet created (flip_estimate_device_bytes: grids, pressure
 * system, particle storage for `particles`), for admission decisions.  No
 * counterpart in the reference, which runs on the host. */
int flip_get_device_bytes(flip_ctx *ctx, long long *bytes);
int flip_estimate_device_bytes(int isize, int jsize, int ksize, int particles, long long *bytes);

/* Many scenes on one GPU: a runtime with `workers` host threads steps
 * contexts concurrently, each on its own stream.  No counterpart in the
 * reference (FluidManager drives one FluidSimulation).
 *   flip_runtime_submit: enqueue `steps` calls of update(dt) on a scene;
 *     requests of one scene run in submission order, requests of different
 *     scenes overlap on the GPU.  A scene must not be used by the caller
 *     while it has requests in flight.
 *   flip_runtime_wait: block until a request is done; its latency (from
 *     submission, queueing included) in ms and its status (that of update).
 *   flip_runtime_update_all: one update(dt) of every listed scene, together;
 *     returns the first error.
 *   flip_runtime_admit: 1 if `bytes` fit in the device's free memory less
 *     the reserve given at creation.
 *   flip_runtime_destroy finishes the submitted requests first. */
typedef struct flip_runtime flip_runtime;
int flip_runtime_create(int workers, long long reserve_bytes, flip_runtime **out);
int flip_runtime_destroy(flip_runtime *rt);
int flip_runtime_submit(flip_runtime *rt, flip_ctx *scene, double dt, int steps, long long *request_id);
int flip_runtime_wait(flip_runtime *rt, long long request_id, double *latency_ms, int *status);
int flip_runtime_update_all(flip_runtime *rt, flip_ctx **scenes, int n, double dt);
int flip_runtime_admit(flip_runtime *rt, long long bytes, int *admitted);
int flip_runtime_pending(flip_runtime *rt, int *queued, int *running);

/* Particle positions in ascending id order, written into caller memory,
 * with no allocation by the library.  No counterpart in the reference: it
 * is the context readback's ordering (flip_get_marker_particle_position_data)
 * for callers that cannot call cudaMalloc, such as hosts whose device memory
 * all comes from their own allocator or pool, or frame loops in which a
 * cudaMalloc's implicit device synchronisation is not acceptable.  Inputs
 * are device arrays of n particles (x, y, z planes and ids, in any order);
 * ids must be distinct and below id_space; an id at or above id_space is
 * skipped.  The output receives packed xyz, the particle with the smallest
 * id first, one row per distinct id below id_space: with m such ids, the
 * first 3*m floats are written and the rest of the buffer is left as it was
 * (m = n when every id is in range).  id_space may be at most
 * FLIP_NOALLOC_MAX_IDS; a larger one is rejected with FLIP_E_OUT_OF_RANGE.
 * The work runs on `stream` (a cudaStream_t; NULL for the default stream) in
 * a device array of about 4 MiB that the library holds until exit on every
 * device that uses it.  The array's address is looked up in the current
 * context on every call (no allocation once the module is loaded); under
 * lazy module loading the first call in a context loads the module, so make
 * it before any stream capture.  Every call shares the array: calls whose
 * work overlaps on the GPU (different streams, or different threads without
 * ordering) race, so order them. */
#define FLIP_NOALLOC_MAX_IDS (1 << 20)
int flip_order_particles_by_id_noalloc(const float *d_px, const float *d_py, const float *d_pz,
                                       const unsigned int *d_ids, int n, int id_space, float *d_out_xyz,
                                       void *stream);

/* Last error message of the calling thread (static storage). */
const char *flip_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* FLIP3D_H */
