/*
 * LBParams.h -- parameters of the D3Q15 MRT model, C++ class API of liblbswim.
 *
 * The struct has the reference's name, field order and types
 * (lbswim/liblbswim/LBParams.h:4-30), so code written against the reference,
 * and its Cython declarations (_lb.pxd:6-17), use it unchanged; it is
 * layout-identical to lbswim_lbparams of lbswim_c.h.
 */
#ifndef LBSWIM_CXX_LBPARAMS_H
#define LBSWIM_CXX_LBPARAMS_H

#ifndef DQ_d
#define DQ_d 3
#endif
#ifndef DQ_q
#define DQ_q 15
#endif

typedef struct LBParams {
  double cs2;                   /* speed of sound, squared */
  double w[DQ_q];               /* quadrature weights */
  double xi[DQ_q][DQ_d];        /* velocities as doubles */
  int ci[DQ_q][DQ_d];           /* velocities as ints */
  double Q[DQ_q][DQ_d][DQ_d];   /* kinetic projector xi_a xi_b - delta_ab cs2 */
  int complement[DQ_q];         /* index of the opposite velocity */
  double norms[DQ_q];           /* normalisers of the modes */
  double mm[DQ_q][DQ_q];        /* mode matrix (rows are the modes) */
  double mmi[DQ_q][DQ_q];       /* its inverse */
  double tau_s;                 /* shear relaxation time */
  double tau_b;                 /* bulk relaxation time */
} LBParams;

#endif
