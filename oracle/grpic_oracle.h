/*
 * CPU oracle for the GR (Kerr-Schild) particle-in-cell path (TEST
 * INFRASTRUCTURE ONLY): a plain-C restatement of the reference's
 * QKerrSchild metric (src/metrics/qkerr_schild.h), GR pusher
 * (src/kernels/pushers/gr.hpp), GR current velocity
 * (src/kernels/currents_deposit.hpp:138-165), GR field kernels
 * (src/kernels/{faraday,ampere,aux_fields}_gr.hpp) and the axis / horizon
 * field boundaries (src/kernels/fields_bcs.hpp:825-868, 1188-1240). Used only
 * by tests/ as the checker of the CUDA path.
 *
 * Grids are 2D (r, theta) with the layout of srpic_oracle.h. Only h = 0
 * (theta = eta) is supported.
 *
 * Precision island: in the single-precision build, particles whose cell
 * satisfies island_lo <= i1 < island_hi (a band of cells around the
 * horizon) run the metric and the push iterations in double, as the product
 * does; the double build runs everything in double.
 */
#ifndef ENTITY_GRPIC_ORACLE_H
#define ENTITY_GRPIC_ORACLE_H

#include "inject_oracle.h"
#include "srpic_oracle.h"

#ifdef __cplusplus
extern "C" {
#endif

/* metric constants in real_t, as QKerrSchild's constructor forms them
 * (qkerr_schild.h:76-94), and the code coordinates of the GR pusher's polar
 * clamp theta in [SMALL_ANGLE_GR, pi - SMALL_ANGLE_GR] (gr.hpp:352-364) */
typedef struct {
  double a, rh, r0, h;
  double chi_min, eta_min, dchi, deta, dchi_inv, deta_inv;
  double x2_small, x2_large;
  int    small_angle;
} orc_qks;

/* theta -> eta and eta -> theta of the angle stretching in real_t
 * (qkerr_schild.h:858-912) */
double orc_qks_theta2eta(double h, double theta);
double orc_qks_eta2theta(double h, double eta);

/* QKerrSchild::convert<2, Ph, Cd> (to_code = 1) or <2, Cd, Ph> (to_code = 0)
 * at n points (qkerr_schild.h:615-649) */
void orc_gr_convert_x2(const orc_qks* q, int to_code, const double* in, int64_t n, double* out);

/* QKerrSchild(res, ext, {a, r0, h}) with ext = [[x1min, x1max], [x2min, x2max]] */
void orc_qks_init(orc_qks* q, int n1, int n2, double x1min, double x1max, double x2min,
                  double x2max, double a, double r0, double h);

/* metric functions at n code-coordinate points x (n x 2, double); out (n x
 * ORC_GR_NQ) in the order: h_11 h_22 h_33 h_13 h11 h22 h33 h13 alpha beta1
 * sqrt_det_h sqrt_det_h_tilde dr_alpha dt_alpha dr_beta1 dt_beta1 dr_h11
 * dr_h22 dr_h33 dr_h13 dt_h11 dt_h22 dt_h33 dt_h13 */
#define ORC_GR_NQ 24
void orc_gr_metric(const orc_qks* q, const double* x, int64_t n, double* out);

/* vector transforms at n points: kind 0 = cov->cntrv, 1 = cntrv->tetrad,
 * 2 = cov->tetrad, 3 = tetrad->cov */
void orc_gr_transform(const orc_qks* q, int kind, const double* x, const double* v, int64_t n,
                      double* out);

/* Pusher_kernel (gr.hpp:664-865): interpolation of D from em and B from em0
 * at shape order `order` (1..3), the leapfrog push, and the particle
 * boundaries (absorb in x1 per absorb[2], axis reflection in x2 per axis[2]).
 * Writes i*_prev/dx*_prev. */
void orc_gr_push(const orc_grid* g, const orc_qks* q, orc_species* sp, const void* em,
                 const void* em0, double dt, double omegaB0, int niter, int order,
                 const int absorb[2], const int axis[2], int island_lo, int island_hi);

/* GR current deposit (currents_deposit.hpp, GR branch, shape order 1):
 * adds into J */
void orc_gr_deposit(const orc_grid* g, const orc_qks* q, const orc_species* sp, void* J,
                    double dt, int island_lo, int island_hi);

/* field kernels; fields are 6-component (D or E in 0..2, B or H in 3..5)
 * Faraday_kernel (faraday_gr.hpp:31-102): Bout = Bin - curl E, over the
 * active cells */
void orc_gr_faraday(const orc_grid* g, const orc_qks* q, const void* Bin, void* Bout,
                    const void* E, double coeff, int axis_min);
/* Ampere_kernel (ampere_gr.hpp:32-101) over i2 in [i2min, i2max + 1); the
 * axis copies of dx1 read Din after the interior update */
void orc_gr_ampere(const orc_grid* g, const orc_qks* q, const void* Din, void* Dout,
                   const void* H, double coeff, int axis_min, int axis_max);
/* CurrentsAmpere_kernel (ampere_gr.hpp:106-176) */
void orc_gr_currents_ampere(const orc_grid* g, const orc_qks* q, void* D, const void* J,
                            double coeff, int axis_min, int axis_max);
/* ComputeAuxE_kernel / ComputeAuxH_kernel (aux_fields_gr.hpp:27-210) over
 * i1 in [i1min - 1, i1max), i2 in [i2min, i2max (+1 with an axis at max)) */
void orc_gr_aux_e(const orc_grid* g, const orc_qks* q, const void* D, const void* B, void* E,
                  int axis_max);
void orc_gr_aux_h(const orc_grid* g, const orc_qks* q, const void* D, const void* B, void* H,
                  int axis_max);
/* TimeAverageDB (all 6 components: f0 = (f0 + f) / 2) and TimeAverageJ
 * (J = (J0 + J) / 2), active cells */
void orc_gr_average_db(const orc_grid* g, const void* f, void* f0);
void orc_gr_average_j(const orc_grid* g, void* J, const void* J0);
/* one pass of grpic::CurrentsFilter: buff <- J, then the 2D axisymmetric
 * stencil of DigitalFilter_kernel with the axis rows (axis_min / axis_max) */
void orc_gr_filter_pass(const orc_grid* g, void* J, void* buff, int axis_min, int axis_max);
/* AxisBoundaries_kernel and HorizonBoundaries_kernel on one field: set_e /
 * set_b select the components (D/E and B/H) */
void orc_gr_field_bcs(const orc_grid* g, void* fld, int set_e, int set_b, int axis_min,
                      int axis_max, int horizon, int nfilter);

/* MATCH at +x1 toward `target` over r in [r_hi - ds, r_hi] (r_lo, r_hi: the
 * grid's radial extent), and the current absorption over the same layer */
void orc_gr_match(const orc_grid* g, const orc_qks* q, void* fld, const void* target, double ds,
                  double r_lo, double r_hi, int set_e, int set_b, int axis_min, int axis_max);
void orc_gr_absorb_currents(const orc_grid* g, const orc_qks* q, void* J, double ds, double r_lo,
                            double r_hi);

/* the uniform Maxwellian pair injection on the QKerrSchild grid
 * (inject_oracle.h for the random numbers): covariant velocities, weight
 * sqrt(det h) / V0 */
int64_t orc_gr_inject_uniform(const orc_grid* g, const orc_qks* q, orc_species* sp1,
                              orc_species* sp2, const orc_inject_params* ip, double V0,
                              int64_t* failures);

#ifdef __cplusplus
}
#endif

#endif /* ENTITY_GRPIC_ORACLE_H */
