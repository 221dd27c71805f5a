// TEST INFRASTRUCTURE: the boundary identifiers and types host/Solver.h uses (the reference's
// BCTypes.h declares the same names: XMIN, XMAX, YMIN, YMAX; Dirichlet, ZeroFlux).
#ifndef DROPIN_BCTYPES_H
#define DROPIN_BCTYPES_H

enum class BoundaryID { XMIN = 0, XMAX = 1, YMIN = 2, YMAX = 3 };
enum class BCType { Dirichlet = 0, ZeroFlux = 1 };

#endif
