// Explicit OpenFOAM polyMesh for the unstructured coupling path: connectivity in compressed rows and the face and
// cell geometry of OpenFOAM's primitiveMesh (face centres and area vectors by a triangle fan about the face's average
// point, cell centres and volumes by pyramids about the average of the face centres).  The reference reads the same
// data through MeshInfo (src/meshinfo.h:20-29: cellCells, cellPoints, points, C, V, Cf, Sf) and mesh.cells()
// (src/geometrictools.cpp:65).  Built on the host (host_poly.cpp), uploaded once per context (capi.cu), read by the
// kernels of poly.cu.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace sdfibm_poly {

struct PolyHostMesh {
    int64_t ncells = 0, npoints = 0, nfaces = 0, ninternal = 0;
    std::vector<double> points;                     // [npoints][3]
    std::vector<int32_t> face_off, face_lab;        // face -> points (stored order)
    std::vector<int32_t> cell_faces_off, cell_faces;  // cell -> faces: owned faces, then neighbour faces (calcCells)
    std::vector<int32_t> cell_pts_off, cell_pts;    // cell -> points, ascending labels (cellPoints)
    std::vector<int32_t> cell_cells_off, cell_cells;  // cell -> face neighbours (cellCells)
    std::vector<double> Cf, Sf, Cc, Vc;             // [nfaces][3], [nfaces][3], [ncells][3], [ncells]
    double bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0};  // bounding box of the points
};

// Builds the mesh from OpenFOAM's polyMesh lists: points [npoints][3], faces as a compact list (face f has the
// labels face_lab[face_off[f] .. face_off[f + 1])), owner [nfaces], neighbour [ninternal].  Returns false with a
// message when the lists are inconsistent (labels out of range, empty faces, cells without faces).
bool build_polymesh(const double* points, int64_t npoints, const int32_t* face_off, const int32_t* face_lab,
                    int64_t nfaces, const int32_t* owner, const int32_t* neighbour, int64_t ninternal,
                    PolyHostMesh& m, std::string& err);

}  // namespace sdfibm_poly
