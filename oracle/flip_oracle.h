// CPU oracle for one FLIP step: a restatement of the reference engine's
// algorithm (jklae/FLIPEngine3D src/engine, FLIP Fluids engine 1.0.9b) for
// the hot path only.  TEST INFRASTRUCTURE: only tests/, the smoke check and
// the CPU-baseline leg of bench.py load it, as the checker.  It is never the
// product path.
//
// Parity pin: tests/test_oracle_vs_reference.py runs the reference engine
// itself (built from its sources by oracle/build_ref.sh) beside this code on
// seeded scenes and tests/test_golden.py checks the committed fixtures that
// tests/golden/make_golden.py produced from it.
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// Buffers filled by orc_update_staged; any pointer may be null.  Face grids
// are (I+1)*J*K (u), I*(J+1)*K (v), I*J*(K+1) (w); cell grids I*J*K; all
// flat index i + nx*(j + ny*k).  Same layout as the reference harness dump.
typedef struct OrcStageDump {
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
} OrcStageDump;

void *orc_create(int isize, int jsize, int ksize, double dx);
void orc_destroy(void *h);
void orc_set_threads(void *h, int n);              // reduction partitions, as setMaxThreadCount
void orc_set_pic_ratio(void *h, double r);
void orc_add_body_force(void *h, double x, double y, double z);
void orc_set_cfl(void *h, int c);
void orc_set_pressure_tol(void *h, double tol);
void orc_set_pressure_maxiter(void *h, int n);
void orc_load_particles(void *h, int n, const float *pos, const float *vel);
void orc_initialize(void *h);
void orc_update(void *h, double dt);
int orc_update_staged(void *h, double dt, OrcStageDump *d);
int orc_num_particles(void *h);
void orc_get_particles(void *h, float *pos, float *vel);
void orc_get_liquid_phi(void *h, float *out);
void orc_get_solid_phi(void *h, float *out);
void orc_get_mac(void *h, float *u, float *v, float *w);
void orc_get_weights(void *h, float *wu, float *wv, float *ww);
void orc_get_near_solid(void *h, int *dims, uint8_t *out);
int orc_last_pcg_iters(void *h);
double orc_last_pcg_error(void *h);
int orc_frame_substeps(void *h);

// The MIC(0) preconditioner alone on a 7-point system over the flagged cells
// (rows in flat cell order; rows7: {diag, +x, +y, +z} per cell).  Returns
// the number of rows.  factor (precondition): {invdiag, L+x, L+y, L+z} floats
// per cell.
int orc_mic0_factor(int I, int J, int K, const uint8_t *fluid, const double *rows7, double *invdiag, double *lower);
int orc_mic0_precondition_f32(int I, int J, int K, const uint8_t *fluid, const float *factor, const float *r,
                              float *z);

#ifdef __cplusplus
}
#endif
