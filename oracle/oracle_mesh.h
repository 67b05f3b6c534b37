// TEST INFRASTRUCTURE ONLY (the oracle): mesh views for the FP64 restatement.
//
// The reference reads its mesh through MeshInfo (src/meshinfo.h:20-29): cellCells, cellPoints, points, C, V, Cf,
// Sf, plus mesh.cells() for the cell->face lists (src/geometrictools.cpp:65).  Two views are given here:
//  * UniformMesh: the implicit single-block hex mesh of sdfibm_mesh_desc with the OpenFOAM ordering conventions
//    (pinned against examples/falling_ellipse/constant/polyMesh of the reference):
//      - point (i,j,k) has label i + (nx+1)(j + (ny+1)k); cellPoints are in ascending label order;
//      - internal faces are upper-triangular (by owner, then neighbour) with the owner's hex-model vertex order;
//      - boundary faces carry the hex-model face of their cell; patches x-min, x-max, y-min, y-max, z-min, z-max;
//      - mesh.cells()[c] = owned faces by face index, then the faces c neighbours, by face index
//        (OpenFOAM primitiveMesh::calcCells), i.e. +x, +y, +z, boundary faces in patch order, -z, -y, -x.
//    Geometry is closed form: x = origin + i*h, C = origin + (i+0.5)*h, V = hx*hy*hz, Cf at the face plane and
//    row centre, Sf = the face's area along its axis.
//  * PolyMesh: an explicit OpenFOAM polyMesh (points / faces / owner / neighbour) with face and cell geometry by
//    OpenFOAM's triangle and pyramid decompositions (primitiveMeshFaceCentresAndAreas, ...CellCentresAndVols).
#pragma once
#include <cstdint>
#include <vector>

#include "../include/sdfibm_cuda.h"
#include "oracle_math.h"

namespace oracle {

struct FaceRef {
    int64_t v[4];  // vertex labels in the face's stored order
    V3 Cf;
    V3 Sf;
};

// Hex vertex slots in ascending label order: 0:(i,j,k) 1:(i+1,j,k) 2:(i,j+1,k) 3:(i+1,j+1,k) 4..7: same at k+1.
// Vertex sequences of the faces of a cell as stored in the mesh (slot indices).
static const int FACE_XMAX_OWN[4] = {1, 3, 7, 5};  // hex model (1 2 6 5)
static const int FACE_YMAX_OWN[4] = {2, 6, 7, 3};  // (3 7 6 2)
static const int FACE_ZMAX_OWN[4] = {4, 5, 7, 6};  // (4 5 6 7)
static const int FACE_XMIN_BND[4] = {0, 4, 6, 2};  // (0 4 7 3)
static const int FACE_YMIN_BND[4] = {0, 1, 5, 4};  // (0 1 5 4)
static const int FACE_ZMIN_BND[4] = {0, 2, 3, 1};  // (0 3 2 1)
static const int FACE_XMIN_NEI[4] = {0, 2, 6, 4};  // x-max face of the lower neighbour seen from this cell
static const int FACE_YMIN_NEI[4] = {0, 4, 5, 1};
static const int FACE_ZMIN_NEI[4] = {0, 1, 3, 2};

struct UniformMesh {
    sdfibm_mesh_desc d;
    int64_t nx, ny, nz, npx, npy;

    explicit UniformMesh(const sdfibm_mesh_desc& m) : d(m), nx(m.nx), ny(m.ny), nz(m.nz), npx(m.nx + 1), npy(m.ny + 1) {}
    int64_t nCells() const { return nx * ny * nz; }
    int64_t nPoints() const { return npx * npy * (nz + 1); }
    void ijk(int64_t c, int64_t& i, int64_t& j, int64_t& k) const {
        i = c % nx; j = (c / nx) % ny; k = c / (nx * ny);
    }
    int64_t cell(int64_t i, int64_t j, int64_t k) const { return i + nx * (j + ny * k); }
    int64_t plabel(int64_t i, int64_t j, int64_t k) const { return i + npx * (j + npy * k); }
    V3 point(int64_t p) const {
        int64_t i = p % npx, j = (p / npx) % npy, k = p / (npx * npy);
        return V3{d.origin[0] + (double)i * d.h[0], d.origin[1] + (double)j * d.h[1], d.origin[2] + (double)k * d.h[2]};
    }
    V3 C(int64_t c) const {
        int64_t i, j, k; ijk(c, i, j, k);
        return V3{d.origin[0] + ((double)i + 0.5) * d.h[0], d.origin[1] + ((double)j + 0.5) * d.h[1],
                  d.origin[2] + ((double)k + 0.5) * d.h[2]};
    }
    double V(int64_t) const { return d.h[0] * d.h[1] * d.h[2]; }
    void cellPoints(int64_t c, int64_t out[8]) const {
        int64_t i, j, k; ijk(c, i, j, k);
        int s = 0;
        for (int dk = 0; dk < 2; ++dk)
            for (int dj = 0; dj < 2; ++dj)
                for (int di = 0; di < 2; ++di) out[s++] = plabel(i + di, j + dj, k + dk);
    }
    // face neighbours (order irrelevant for the enumeration result)
    int cellCells(int64_t c, int64_t out[6]) const {
        int64_t i, j, k; ijk(c, i, j, k);
        int n = 0;
        if (i + 1 < nx) out[n++] = c + 1;
        if (j + 1 < ny) out[n++] = c + nx;
        if (k + 1 < nz) out[n++] = c + nx * ny;
        if (k > 0) out[n++] = c - nx * ny;
        if (j > 0) out[n++] = c - nx;
        if (i > 0) out[n++] = c - 1;
        return n;
    }
    // mesh.cells()[c] in OpenFOAM order, with vertex sequences and closed-form Cf, Sf
    int cellFaces(int64_t c, FaceRef out[6]) const {
        int64_t i, j, k; ijk(c, i, j, k);
        int64_t v[8]; cellPoints(c, v);
        const double* o = d.origin; const double* h = d.h;
        const double xc = o[0] + ((double)i + 0.5) * h[0], yc = o[1] + ((double)j + 0.5) * h[1],
                     zc = o[2] + ((double)k + 0.5) * h[2];
        const double xlo = o[0] + (double)i * h[0], xhi = o[0] + (double)(i + 1) * h[0];
        const double ylo = o[1] + (double)j * h[1], yhi = o[1] + (double)(j + 1) * h[1];
        const double zlo = o[2] + (double)k * h[2], zhi = o[2] + (double)(k + 1) * h[2];
        const V3 Sx{h[1] * h[2], 0, 0}, Sy{0, h[0] * h[2], 0}, Sz{0, 0, h[0] * h[1]};
        int n = 0;
        auto put = [&](const int* slots, const V3& cf, const V3& sf) {
            for (int q = 0; q < 4; ++q) out[n].v[q] = v[slots[q]];
            out[n].Cf = cf; out[n].Sf = sf; ++n;
        };
        if (i + 1 < nx) put(FACE_XMAX_OWN, V3{xhi, yc, zc}, Sx);
        if (j + 1 < ny) put(FACE_YMAX_OWN, V3{xc, yhi, zc}, Sy);
        if (k + 1 < nz) put(FACE_ZMAX_OWN, V3{xc, yc, zhi}, Sz);
        if (i == 0) put(FACE_XMIN_BND, V3{xlo, yc, zc}, Sx);
        if (i == nx - 1) put(FACE_XMAX_OWN, V3{xhi, yc, zc}, Sx);
        if (j == 0) put(FACE_YMIN_BND, V3{xc, ylo, zc}, Sy);
        if (j == ny - 1) put(FACE_YMAX_OWN, V3{xc, yhi, zc}, Sy);
        if (k == 0) put(FACE_ZMIN_BND, V3{xc, yc, zlo}, Sz);
        if (k == nz - 1) put(FACE_ZMAX_OWN, V3{xc, yc, zhi}, Sz);
        if (k > 0) put(FACE_ZMIN_NEI, V3{xc, yc, zlo}, Sz);
        if (j > 0) put(FACE_YMIN_NEI, V3{xc, ylo, zc}, Sy);
        if (i > 0) put(FACE_XMIN_NEI, V3{xlo, yc, zc}, Sx);
        return n;
    }
    V3 boundsMin() const { return point(0); }
    V3 boundsMax() const { return point(plabel(nx, ny, nz)); }
};

// Explicit OpenFOAM polyMesh.  faces: offsets (nFaces+1) + labels; owner (nFaces), neighbour (nInternal).
struct PolyMesh {
    std::vector<V3> points;
    std::vector<std::vector<int64_t>> faces;
    std::vector<int64_t> owner, neighbour;
    std::vector<std::vector<int64_t>> cells, cellPointsL, cellCellsL;
    std::vector<V3> Cf, Sf, Cc;
    std::vector<double> Vc;
    V3 bmin, bmax;

    int64_t nCells() const { return (int64_t)cells.size(); }

    void build() {
        int64_t nc = 0;
        for (int64_t o : owner) nc = std::max(nc, o + 1);
        for (int64_t nb : neighbour) nc = std::max(nc, nb + 1);
        // primitiveMesh::calcCells: owner loop then neighbour loop
        cells.assign(nc, {});
        for (size_t f = 0; f < owner.size(); ++f) cells[owner[f]].push_back((int64_t)f);
        for (size_t f = 0; f < neighbour.size(); ++f) cells[neighbour[f]].push_back((int64_t)f);
        // face centres and areas (triangle fan about the face average point)
        size_t nf = faces.size();
        Cf.resize(nf); Sf.resize(nf);
        for (size_t f = 0; f < nf; ++f) {
            const auto& fv = faces[f];
            size_t np = fv.size();
            V3 fc = points[fv[0]];
            for (size_t q = 1; q < np; ++q) fc = fc + points[fv[q]];
            fc = fc / (double)np;
            V3 sumN{0, 0, 0}, sumAc{0, 0, 0};
            double sumA = 0.0;
            for (size_t q = 0; q < np; ++q) {
                const V3& pq = points[fv[q]];
                const V3& nxt = points[fv[(q + 1) % np]];
                V3 c = pq + nxt + fc;
                V3 nrm = cross(nxt - pq, fc - pq);
                double a = mag(nrm);
                sumN = sumN + nrm; sumA += a; sumAc = sumAc + a * c;
            }
            if (sumA < 1e-150) { Cf[f] = fc; Sf[f] = V3{0, 0, 0}; }
            else { Cf[f] = (1.0 / 3.0) * sumAc / sumA; Sf[f] = 0.5 * sumN; }
        }
        // cell centres and volumes (pyramids about the average of face centres)
        std::vector<V3> cEst(nc, V3{0, 0, 0});
        std::vector<int> ncf(nc, 0);
        for (size_t f = 0; f < owner.size(); ++f) { cEst[owner[f]] += Cf[f]; ncf[owner[f]] += 1; }
        for (size_t f = 0; f < neighbour.size(); ++f) { cEst[neighbour[f]] += Cf[f]; ncf[neighbour[f]] += 1; }
        for (int64_t c = 0; c < nc; ++c) cEst[c] = cEst[c] / (double)ncf[c];
        Cc.assign(nc, V3{0, 0, 0}); Vc.assign(nc, 0.0);
        for (size_t f = 0; f < owner.size(); ++f) {
            int64_t c = owner[f];
            double pyr3 = dot(Sf[f], Cf[f] - cEst[c]);
            V3 pc = (3.0 / 4.0) * Cf[f] + (1.0 / 4.0) * cEst[c];
            Cc[c] += pyr3 * pc; Vc[c] += pyr3;
        }
        for (size_t f = 0; f < neighbour.size(); ++f) {
            int64_t c = neighbour[f];
            double pyr3 = dot(Sf[f], cEst[c] - Cf[f]);
            V3 pc = (3.0 / 4.0) * Cf[f] + (1.0 / 4.0) * cEst[c];
            Cc[c] += pyr3 * pc; Vc[c] += pyr3;
        }
        for (int64_t c = 0; c < nc; ++c) {
            if (std::fabs(Vc[c]) > 1e-300) Cc[c] = Cc[c] / Vc[c]; else Cc[c] = cEst[c];
            Vc[c] *= (1.0 / 3.0);
        }
        // cellPoints ascending (invertManyToMany of pointCells), cellCells
        cellPointsL.assign(nc, {});
        std::vector<std::vector<int64_t>> pointCells(points.size());
        for (int64_t c = 0; c < nc; ++c) {
            std::vector<int64_t> pts;
            for (int64_t f : cells[c]) for (int64_t p : faces[f]) pts.push_back(p);
            std::sort(pts.begin(), pts.end());
            pts.erase(std::unique(pts.begin(), pts.end()), pts.end());
            for (int64_t p : pts) pointCells[p].push_back(c);
        }
        for (size_t p = 0; p < points.size(); ++p)
            for (int64_t c : pointCells[p]) cellPointsL[c].push_back((int64_t)p);
        cellCellsL.assign(nc, {});
        for (size_t f = 0; f < neighbour.size(); ++f) {
            cellCellsL[owner[f]].push_back(neighbour[f]);
            cellCellsL[neighbour[f]].push_back(owner[f]);
        }
        bmin = bmax = points[0];
        for (const V3& p : points) {
            bmin.x = std::min(bmin.x, p.x); bmin.y = std::min(bmin.y, p.y); bmin.z = std::min(bmin.z, p.z);
            bmax.x = std::max(bmax.x, p.x); bmax.y = std::max(bmax.y, p.y); bmax.z = std::max(bmax.z, p.z);
        }
    }
};

}  // namespace oracle
