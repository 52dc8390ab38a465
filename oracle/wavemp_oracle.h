/* wavemp_oracle.h -- CPU restatement of the reference's per-stage RHS (test infrastructure only).
 * See wavemp_oracle.c for the correspondence with the reference scripts. */
#ifndef WAVEMP_ORACLE_H
#define WAVEMP_ORACLE_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_SC = 0, ORC_M10 = 1 };          /* scheme variant (which reference script) */
enum { ORC_SHIPPED = 0, ORC_MP5C6 = 1 };   /* reconstruction: MUSCL+central-4 or MP5+central-6 */

typedef struct {
    double g1, p1, g2, p2; /* stiffened-gas gamma / p_inf of fluid 1 and fluid 2 */
    double dx, dy, cfl;
    int variant, recon;
    int bc[4];  /* x-low, x-high, y-low, y-high: 0 transmissive, 1 slip wall */
    int repair; /* emergency admissibility repair after every stage */
} orc_params;

enum {
    ORC_FN_MP5_UL = 0, ORC_FN_MP5_UR, ORC_FN_CENTRAL6, ORC_FN_MUSCL_UL, ORC_FN_MUSCL_UR,
    ORC_FN_THINC_UL, ORC_FN_THINC_UR, ORC_FN_CATOR2, ORC_FN_MM4, ORC_FN_MM2, ORC_FN_EOS,
    ORC_FN_HLLC_X, ORC_FN_HLLC_Y, ORC_FN_EIGEN, ORC_FN_PPLIM, ORC_FN_THETA
};

void orc_cons_to_prim(const orc_params *P, int nxg, int nyg, double *ar1, double *ar2, double *ru,
                      double *rv, double *E, double *al, double *u_p, double *v_p, double *p_p);
void orc_ducros(int nxg, int nyg, const double *u_p, const double *v_p, const double *p_p,
                double *sigma_x, double *sigma_y);
void orc_enforce_admissible(const orc_params *P, int nxg, int nyg, double *ar1, double *ar2,
                            double *ru, double *rv, double *E, double *al);
void orc_face_flux(const orc_params *P, int dir, int nx, int ny, int g, const double *const cell[6],
                   const double *sigma, double *const out[7]);
void orc_face_flux_low(const orc_params *P, int dir, int nx, int ny, int g,
                       const double *const cell[6], double *const out[7]);
void orc_cell_theta(const orc_params *P, int nx, int ny, int g, const double *const q[6],
                    const double *al_prim, const double *const fh[7], const double *const gh[7],
                    const double *const fl[7], const double *const gl[7], double *theta_cell,
                    double dt, int stage);
void orc_blend(int dir, int nx, int ny, int g, double *const fh[7], const double *const fl[7],
               const double *theta_cell);
void orc_rk3(const orc_params *P, int nx, int ny, int g, const double *const q_old[6],
             double *const q[6], const double *al_prim, const double *const fx[7],
             const double *const gy[7], double dt, double alpha, double beta);
void orc_apply_bc(const int bc[4], int nx, int ny, int g, double *const f9[9]);
double orc_get_dt(const orc_params *P, int nx, int ny, int g, const double *ar1, const double *ar2,
                  const double *u_p, const double *v_p, const double *p_p, const double *al);
size_t orc_workspace_doubles(int nx, int ny, int g);
void orc_stage(const orc_params *P, int nx, int ny, int g, double *const f10[10],
               const double *const q_old[6], double *ws, double dt, double alpha, double beta);
void orc_steps(const orc_params *P, int nx, int ny, int g, double *const f10[10], double *ws,
               int nsteps, double *dt);
void orc_init_sequence(const orc_params *P, int nx, int ny, int g, double *const f10[10]);
int orc_unit(const orc_params *P, int fn, long n, const double *in, int in_stride, double *out,
             int out_stride);

#ifdef __cplusplus
}
#endif
#endif
