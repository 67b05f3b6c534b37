// Host-side construction of an explicit polyMesh (poly.hpp).  Compiled with -ffp-contract=off: every FP64 operation
// of the geometry is a separate rounding, in OpenFOAM's order, so the cell centres that decide the centre-inside test
// are the same numbers on every host.
#include "poly.hpp"

#include <algorithm>
#include <cmath>

namespace sdfibm_poly {

namespace {
struct V {
    double x, y, z;
};
inline V add(const V& a, const V& b) { return V{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V sub(const V& a, const V& b) { return V{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V scale(double s, const V& a) { return V{s * a.x, s * a.y, s * a.z}; }
inline V divide(const V& a, double s) { return V{a.x / s, a.y / s, a.z / s}; }
inline double dotp(const V& a, const V& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V crossp(const V& a, const V& b) { return V{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double norm(const V& a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
}  // namespace

bool build_polymesh(const double* points, int64_t npoints, const int32_t* face_off, const int32_t* face_lab,
                    int64_t nfaces, const int32_t* owner, const int32_t* neighbour, int64_t ninternal,
                    PolyHostMesh& m, std::string& err) {
    if (!points || !face_off || !face_lab || !owner || (ninternal > 0 && !neighbour) || npoints <= 0 || nfaces <= 0 ||
        ninternal < 0 || ninternal > nfaces || npoints >= (1ll << 31) || nfaces >= (1ll << 31)) {
        err = "polyMesh: bad list sizes";
        return false;
    }
    m = PolyHostMesh();
    m.npoints = npoints;
    m.nfaces = nfaces;
    m.ninternal = ninternal;
    m.points.assign(points, points + 3 * npoints);
    if (face_off[0] != 0) { err = "polyMesh: face offsets do not start at 0"; return false; }
    for (int64_t f = 0; f < nfaces; ++f)
        if (face_off[f + 1] - face_off[f] < 3) { err = "polyMesh: a face has fewer than 3 points"; return false; }
    const int64_t nlab = face_off[nfaces];
    for (int64_t q = 0; q < nlab; ++q)
        if (face_lab[q] < 0 || face_lab[q] >= npoints) { err = "polyMesh: point label out of range"; return false; }
    m.face_off.assign(face_off, face_off + nfaces + 1);
    m.face_lab.assign(face_lab, face_lab + nlab);
    int64_t nc = 0;
    for (int64_t f = 0; f < nfaces; ++f) {
        if (owner[f] < 0) { err = "polyMesh: negative owner"; return false; }
        nc = std::max<int64_t>(nc, (int64_t)owner[f] + 1);
    }
    for (int64_t f = 0; f < ninternal; ++f) {
        if (neighbour[f] < 0) { err = "polyMesh: negative neighbour"; return false; }
        nc = std::max<int64_t>(nc, (int64_t)neighbour[f] + 1);
    }
    if (nc >= (1ll << 31)) { err = "polyMesh: too many cells"; return false; }
    m.ncells = nc;
    // cell -> faces (primitiveMesh::calcCells: the owner loop, then the neighbour loop)
    std::vector<int32_t> cnt(nc + 1, 0);
    for (int64_t f = 0; f < nfaces; ++f) ++cnt[owner[f] + 1];
    for (int64_t f = 0; f < ninternal; ++f) ++cnt[neighbour[f] + 1];
    m.cell_faces_off.assign(nc + 1, 0);
    for (int64_t c = 0; c < nc; ++c) m.cell_faces_off[c + 1] = m.cell_faces_off[c] + cnt[c + 1];
    m.cell_faces.assign(m.cell_faces_off[nc], 0);
    std::vector<int32_t> cur(m.cell_faces_off.begin(), m.cell_faces_off.end() - 1);
    for (int64_t f = 0; f < nfaces; ++f) m.cell_faces[cur[owner[f]]++] = (int32_t)f;
    for (int64_t f = 0; f < ninternal; ++f) m.cell_faces[cur[neighbour[f]]++] = (int32_t)f;
    for (int64_t c = 0; c < nc; ++c)
        if (m.cell_faces_off[c + 1] == m.cell_faces_off[c]) { err = "polyMesh: a cell has no faces"; return false; }
    auto P = [&](int64_t p) { return V{points[3 * p], points[3 * p + 1], points[3 * p + 2]}; };
    // face centres and area vectors: triangles about the average point (primitiveMeshFaceCentresAndAreas)
    m.Cf.assign(3 * nfaces, 0.0);
    m.Sf.assign(3 * nfaces, 0.0);
    for (int64_t f = 0; f < nfaces; ++f) {
        const int32_t b = face_off[f], np = face_off[f + 1] - b;
        V fc = P(face_lab[b]);
        for (int q = 1; q < np; ++q) fc = add(fc, P(face_lab[b + q]));
        fc = divide(fc, (double)np);
        V sumN{0, 0, 0}, sumAc{0, 0, 0};
        double sumA = 0.0;
        for (int q = 0; q < np; ++q) {
            const V pq = P(face_lab[b + q]);
            const V nxt = P(face_lab[b + (q + 1) % np]);
            const V c = add(add(pq, nxt), fc);
            const V nrm = crossp(sub(nxt, pq), sub(fc, pq));
            const double a = norm(nrm);
            sumN = add(sumN, nrm);
            sumA += a;
            sumAc = add(sumAc, scale(a, c));
        }
        V cf, sf;
        if (sumA < 1e-150) {
            cf = fc;
            sf = V{0, 0, 0};
        } else {
            cf = divide(scale(1.0 / 3.0, sumAc), sumA);
            sf = scale(0.5, sumN);
        }
        m.Cf[3 * f] = cf.x; m.Cf[3 * f + 1] = cf.y; m.Cf[3 * f + 2] = cf.z;
        m.Sf[3 * f] = sf.x; m.Sf[3 * f + 1] = sf.y; m.Sf[3 * f + 2] = sf.z;
    }
    auto CF = [&](int64_t f) { return V{m.Cf[3 * f], m.Cf[3 * f + 1], m.Cf[3 * f + 2]}; };
    auto SF = [&](int64_t f) { return V{m.Sf[3 * f], m.Sf[3 * f + 1], m.Sf[3 * f + 2]}; };
    // cell centres and volumes: pyramids about the average of the face centres (primitiveMeshCellCentresAndVols)
    std::vector<V> cEst(nc, V{0, 0, 0});
    std::vector<int> ncf(nc, 0);
    for (int64_t f = 0; f < nfaces; ++f) { cEst[owner[f]] = add(cEst[owner[f]], CF(f)); ncf[owner[f]] += 1; }
    for (int64_t f = 0; f < ninternal; ++f) {
        cEst[neighbour[f]] = add(cEst[neighbour[f]], CF(f));
        ncf[neighbour[f]] += 1;
    }
    for (int64_t c = 0; c < nc; ++c) cEst[c] = divide(cEst[c], (double)ncf[c]);
    std::vector<V> cc(nc, V{0, 0, 0});
    std::vector<double> vc(nc, 0.0);
    for (int64_t f = 0; f < nfaces; ++f) {
        const int64_t c = owner[f];
        const double pyr3 = dotp(SF(f), sub(CF(f), cEst[c]));
        const V pc = add(scale(3.0 / 4.0, CF(f)), scale(1.0 / 4.0, cEst[c]));
        cc[c] = add(cc[c], scale(pyr3, pc));
        vc[c] += pyr3;
    }
    for (int64_t f = 0; f < ninternal; ++f) {
        const int64_t c = neighbour[f];
        const double pyr3 = dotp(SF(f), sub(cEst[c], CF(f)));
        const V pc = add(scale(3.0 / 4.0, CF(f)), scale(1.0 / 4.0, cEst[c]));
        cc[c] = add(cc[c], scale(pyr3, pc));
        vc[c] += pyr3;
    }
    m.Cc.assign(3 * nc, 0.0);
    m.Vc.assign(nc, 0.0);
    for (int64_t c = 0; c < nc; ++c) {
        const V x = std::fabs(vc[c]) > 1e-300 ? divide(cc[c], vc[c]) : cEst[c];
        m.Cc[3 * c] = x.x; m.Cc[3 * c + 1] = x.y; m.Cc[3 * c + 2] = x.z;
        m.Vc[c] = vc[c] * (1.0 / 3.0);
    }
    // cell -> points in ascending label order (cellPoints), cell -> face neighbours (cellCells)
    m.cell_pts_off.assign(nc + 1, 0);
    std::vector<int32_t> pts;
    std::vector<std::vector<int32_t>> cp(nc);
    for (int64_t c = 0; c < nc; ++c) {
        pts.clear();
        for (int32_t q = m.cell_faces_off[c]; q < m.cell_faces_off[c + 1]; ++q) {
            const int32_t f = m.cell_faces[q];
            for (int32_t r = face_off[f]; r < face_off[f + 1]; ++r) pts.push_back(face_lab[r]);
        }
        std::sort(pts.begin(), pts.end());
        pts.erase(std::unique(pts.begin(), pts.end()), pts.end());
        cp[c] = pts;
        m.cell_pts_off[c + 1] = m.cell_pts_off[c] + (int32_t)pts.size();
    }
    m.cell_pts.reserve(m.cell_pts_off[nc]);
    for (int64_t c = 0; c < nc; ++c) m.cell_pts.insert(m.cell_pts.end(), cp[c].begin(), cp[c].end());
    std::vector<int32_t> ncc(nc + 1, 0);
    for (int64_t f = 0; f < ninternal; ++f) { ++ncc[owner[f] + 1]; ++ncc[neighbour[f] + 1]; }
    m.cell_cells_off.assign(nc + 1, 0);
    for (int64_t c = 0; c < nc; ++c) m.cell_cells_off[c + 1] = m.cell_cells_off[c] + ncc[c + 1];
    m.cell_cells.assign(m.cell_cells_off[nc], 0);
    std::vector<int32_t> cc2(m.cell_cells_off.begin(), m.cell_cells_off.end() - 1);
    for (int64_t f = 0; f < ninternal; ++f) {
        m.cell_cells[cc2[owner[f]]++] = neighbour[f];
        m.cell_cells[cc2[neighbour[f]]++] = owner[f];
    }
    for (int a = 0; a < 3; ++a) { m.bmin[a] = points[a]; m.bmax[a] = points[a]; }
    for (int64_t p = 0; p < npoints; ++p)
        for (int a = 0; a < 3; ++a) {
            m.bmin[a] = std::min(m.bmin[a], points[3 * p + a]);
            m.bmax[a] = std::max(m.bmax[a], points[3 * p + a]);
        }
    return true;
}

}  // namespace sdfibm_poly
