// VTK XML PolyData dumps of a detection pass (see cc_vtk.cpp).
#pragma once

namespace ccg {

// n_elems elements with 3 point ids each (a bond's third is -1), indexing
// pos / imp (3 doubles per point) and num (contributions per point).
bool write_vtp(const char* path, int n_elems, const int* ev, const double* pos, const double* imp, const double* num);

}  // namespace ccg
