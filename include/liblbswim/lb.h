/* lb.h -- the header the reference's Cython declarations name for the lattice
 * (lbswim/liblbswim/lb.h, _lb.pxd:3); C++ class API of liblbswim. */
#ifndef LBSWIM_CXX_LB_H
#define LBSWIM_CXX_LB_H

#include "Lattice.h"

#endif
