// Periodic-cell preparation for neighbour search: axis reduction, wrapping
// of positions and the list of lattice translations, as NeighborCell
// (src/pypolymlp/cxx/src/compute/neighbor_cell.cpp:11-253).  Computed on the
// host in IEEE double with the reference's operation order (this file must
// be compiled with -ffp-contract=off) so that the device pair search sees
// bit-identical translation vectors and positions.
#pragma once

#include <array>
#include <vector>

namespace pg {

struct CellTranslations {
    std::vector<std::array<double, 3>> trans;   // lattice translations (Cartesian)
    std::vector<std::array<int, 3>> tn;         // their integer coefficients on the (reduced) axis
    std::vector<std::array<double, 3>> pos;     // positions after optional wrapping
    double axis[3][3];                          // the (reduced) axis, [row][col], columns are lattice vectors
};

// axis: row-major 3x3 with lattice vectors as columns; pos: n x 3 Cartesian.
CellTranslations cell_translations(const double* axis, const double* pos, int n, double cutoff);

}  // namespace pg
