/*
 * d3q15.h -- D3Q15 velocity set constants, C++ class API of liblbswim.
 *
 * The macro names of the reference's d3q15.h:4-32 (dimensions, axis and mode
 * indices), and LatticeEigenSet (d3q15.c:2), which fills every table of an
 * LBParams from the D3Q15 definitions through the library.
 */
#ifndef LBSWIM_CXX_D3Q15_H
#define LBSWIM_CXX_D3Q15_H

#define DQ_d 3
#define DQ_q 15

/* dimensions */
#define DQ_X 0
#define DQ_Y 1
#define DQ_Z 2

/* mode indices (rows of LBParams::mm) */
#define DQ_rho 0
#define DQ_momX 1
#define DQ_momY 2
#define DQ_momZ 3
#define DQ_SXX 4
#define DQ_SXY 5
#define DQ_SXZ 6
#define DQ_SYY 7
#define DQ_SYZ 8
#define DQ_SZZ 9
#define DQ_chi1 10
#define DQ_jchi1X 11
#define DQ_jchi1Y 12
#define DQ_jchi1Z 13
#define DQ_chi2 14
#define DQ_mom(dim) (1 + (dim))

#include "LBParams.h"
#include "lbswim_c.h"

static_assert(sizeof(LBParams) == sizeof(lbswim_lbparams), "LBParams layout");

/* Fills cs2, w, xi, ci, Q, complement, norms, mm and mmi; keeps tau_s, tau_b. */
inline void LatticeEigenSet(LBParams* lat) {
  lbswim_lbparams_fill(reinterpret_cast<lbswim_lbparams*>(lat));
}

#endif
