// microstructure.hpp -- element phase from the element centroid, for the reference's 13 micro types.
#pragma once

namespace mgb {

// get_elem_type (micropp.cpp:338-544): phase (0 matrix, 1 or 2 inclusion) of element (ex, ey, ez) of a unit
// cube with element sizes dx, dy, dz; -1 for an unknown micro_type.
int micro_elem_type(int micro_type, const double geo[4], int ex, int ey, int ez, double dx, double dy, double dz);

}  // namespace mgb
