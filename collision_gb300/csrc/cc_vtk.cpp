// Debugging dumps of a detection pass as VTK XML PolyData (.vtp), the
// equivalent of the reference's vtkplotVectorSurface (vtk.cpp:14-93), which
// updateAverageVelocity calls on every pass under the "CollisionImpulse"
// debugging flag (dcollid.cpp:684-693): the surface at x_old + dt*avgVel
// before the pass's impulses are applied, each point's accumulated impulse
// (CollsnImpulse) and, per element, red where one of its points was hit in
// the pass and green elsewhere (CollsnRegion). Points are numbered in order
// of first appearance in the element list and only element points are
// written, as there. Written in the ASCII form of the format, without the
// VTK library.
#include "cc_vtk.h"

#include <cstdio>
#include <vector>

namespace ccg {

bool write_vtp(const char* path, int n_elems, const int* ev, const double* pos, const double* imp,
               const double* num) {
    FILE* f = std::fopen(path, "w");
    if (!f) return false;
    // number the points of the elements by first appearance
    std::vector<int> id_of;
    std::vector<int> order;
    int maxp = -1;
    for (int e = 0; e < n_elems; ++e)
        for (int k = 0; k < 3; ++k) maxp = ev[3 * e + k] > maxp ? ev[3 * e + k] : maxp;
    id_of.assign((size_t)(maxp + 1), -1);
    for (int e = 0; e < n_elems; ++e)
        for (int k = 0; k < 3; ++k) {
            int p = ev[3 * e + k];
            if (p < 0 || id_of[p] >= 0) continue;
            id_of[p] = (int)order.size();
            order.push_back(p);
        }
    std::fprintf(f, "<?xml version=\"1.0\"?>\n");
    std::fprintf(f, "<VTKFile type=\"PolyData\" version=\"0.1\" byte_order=\"LittleEndian\">\n<PolyData>\n");
    std::fprintf(f,
                 "<Piece NumberOfPoints=\"%d\" NumberOfVerts=\"0\" NumberOfLines=\"0\" NumberOfStrips=\"0\" "
                 "NumberOfPolys=\"%d\">\n",
                 (int)order.size(), n_elems);
    std::fprintf(f, "<PointData Vectors=\"CollsnImpulse\">\n");
    std::fprintf(f, "<DataArray type=\"Float32\" Name=\"CollsnImpulse\" NumberOfComponents=\"3\" format=\"ascii\">\n");
    for (int p : order) std::fprintf(f, "%.9g %.9g %.9g\n", imp[3 * p], imp[3 * p + 1], imp[3 * p + 2]);
    std::fprintf(f, "</DataArray>\n</PointData>\n");
    std::fprintf(f, "<CellData Scalars=\"CollsnRegion\">\n");
    std::fprintf(f, "<DataArray type=\"UInt8\" Name=\"CollsnRegion\" NumberOfComponents=\"3\" format=\"ascii\">\n");
    for (int e = 0; e < n_elems; ++e) {
        bool hit = false;
        for (int k = 0; k < 3; ++k) {
            int p = ev[3 * e + k];
            if (p >= 0 && num[p] > 0) hit = true;
        }
        std::fprintf(f, hit ? "255 0 0\n" : "0 255 0\n");
    }
    std::fprintf(f, "</DataArray>\n</CellData>\n");
    std::fprintf(f, "<Points>\n<DataArray type=\"Float32\" NumberOfComponents=\"3\" format=\"ascii\">\n");
    for (int p : order) std::fprintf(f, "%.9g %.9g %.9g\n", pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]);
    std::fprintf(f, "</DataArray>\n</Points>\n");
    std::fprintf(f, "<Polys>\n<DataArray type=\"Int32\" Name=\"connectivity\" format=\"ascii\">\n");
    for (int e = 0; e < n_elems; ++e) {
        int np = ev[3 * e + 2] >= 0 ? 3 : 2;
        for (int k = 0; k < np; ++k) std::fprintf(f, "%d ", id_of[ev[3 * e + k]]);
        std::fprintf(f, "\n");
    }
    std::fprintf(f, "</DataArray>\n<DataArray type=\"Int32\" Name=\"offsets\" format=\"ascii\">\n");
    long long off = 0;
    for (int e = 0; e < n_elems; ++e) {
        off += ev[3 * e + 2] >= 0 ? 3 : 2;
        std::fprintf(f, "%lld\n", off);
    }
    std::fprintf(f, "</DataArray>\n</Polys>\n</Piece>\n</PolyData>\n</VTKFile>\n");
    return std::fclose(f) == 0;
}

}  // namespace ccg
