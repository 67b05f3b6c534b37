"""Test helper: OpenFOAM polyMesh lists of structured hex meshes (the tests of the unstructured-mesh path).

block_mesh() builds the mesh of a blockMeshDict made of hex blocks with straight edges and simpleGrading:
  * points block after block, each block's points i fastest, then j, then k, a point shared with an earlier block
    keeping that block's label (blockMesh's merge); coordinates by interpolation between the block's corner vertices
    at the graded parameters, the divisions of a direction with expansion ratio R over n cells being
    (1 - r^i) / (1 - r^n) with r = R^(1 / (n - 1)) (cell sizes in geometric progression, last / first = R);
  * cells block after block, i fastest;
  * faces with the OpenFOAM hex model's outward vertex order of their owner cell (the lower cell label):
    x-min (0 4 7 3), x-max (1 2 6 5), y-min (0 1 5 4), y-max (3 7 6 2), z-min (0 3 2 1), z-max (4 5 6 7);
    internal faces first, ordered by owner then neighbour, then the boundary faces by owner.
jiggle() moves the interior points at random (general hexahedra with non-planar faces).
"""
import numpy as np

# outward faces of the hex model (vertex 0 (0,0,0), 1 (1,0,0), 2 (1,1,0), 3 (0,1,0), 4..7 the same at z = 1)
HEX_FACES = [(0, 4, 7, 3), (1, 2, 6, 5), (0, 1, 5, 4), (3, 7, 6, 2), (0, 3, 2, 1), (4, 5, 6, 7)]


def divisions(n, R):
    if n <= 1 or R == 1.0:
        return np.arange(n + 1, dtype=np.float64) / n
    r = R ** (1.0 / (n - 1))
    return (1.0 - r ** np.arange(n + 1, dtype=np.float64)) / (1.0 - r ** n)


def block_mesh(vertices, hexes, counts, grading):
    """(points [P, 3], face_off [F + 1], face_lab, owner [F], neighbour [F_int], ncells)."""
    vertices = np.asarray(vertices, np.float64)
    pts, index = [], {}
    cells = []
    for hx, (nx, ny, nz), (gx, gy, gz) in zip(hexes, counts, grading):
        v = vertices[list(hx)]           # hex-model corners
        lx, ly, lz = divisions(nx, gx), divisions(ny, gy), divisions(nz, gz)
        labels = np.zeros((nz + 1, ny + 1, nx + 1), dtype=np.int64)
        for k in range(nz + 1):
            for j in range(ny + 1):
                for i in range(nx + 1):
                    a, b, c = lx[i], ly[j], lz[k]
                    # trilinear interpolation of the 8 corners (exact on the block's straight edges)
                    p = ((1 - a) * (1 - b) * (1 - c) * v[0] + a * (1 - b) * (1 - c) * v[1] + a * b * (1 - c) * v[2] +
                         (1 - a) * b * (1 - c) * v[3] + (1 - a) * (1 - b) * c * v[4] + a * (1 - b) * c * v[5] +
                         a * b * c * v[6] + (1 - a) * b * c * v[7])
                    key = tuple(np.round(p, 9))
                    if key not in index:
                        index[key] = len(pts)
                        pts.append(p)
                    labels[k, j, i] = index[key]
        for k in range(nz):
            for j in range(ny):
                for i in range(nx):
                    cells.append([labels[k, j, i], labels[k, j, i + 1], labels[k, j + 1, i + 1], labels[k, j + 1, i],
                                  labels[k + 1, j, i], labels[k + 1, j, i + 1], labels[k + 1, j + 1, i + 1],
                                  labels[k + 1, j + 1, i]])
    faces = {}
    for c, cv in enumerate(cells):
        for f in HEX_FACES:
            fv = tuple(cv[q] for q in f)
            key = tuple(sorted(fv))
            if key in faces:
                faces[key][2] = c      # the second cell is the neighbour (higher label)
            else:
                faces[key] = [fv, c, -1]
    internal = sorted((o, n, fv) for fv, o, n in faces.values() if n >= 0)
    boundary = sorted((o, fv) for fv, o, n in faces.values() if n < 0)
    flist = [fv for _, _, fv in internal] + [fv for _, fv in boundary]
    owner = np.array([o for o, _, _ in internal] + [o for o, _ in boundary], np.int32)
    neighbour = np.array([n for _, n, _ in internal], np.int32)
    face_off = np.zeros(len(flist) + 1, np.int32)
    face_off[1:] = np.cumsum([len(f) for f in flist])
    face_lab = np.array([p for f in flist for p in f], np.int32)
    return np.array(pts), face_off, face_lab, owner, neighbour, len(cells)


def uniform_block(n, origin, h):
    """One block of n[0] x n[1] x n[2] equal cells of size h from origin."""
    o = np.asarray(origin, np.float64)
    L = np.asarray(n, np.float64) * np.asarray(h, np.float64)
    corners = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]],
                       np.float64)
    verts = o + corners * L
    return block_mesh(verts, [list(range(8))], [list(n)], [[1.0, 1.0, 1.0]])


def jiggle(points, amplitude, seed, keep_z=False):
    """Interior points moved by up to `amplitude` per axis (boundary points stay on the box)."""
    p = np.array(points, np.float64)
    lo, hi = p.min(0), p.max(0)
    inner = np.all((p > lo + 1e-9) & (p < hi - 1e-9), axis=1) if not keep_z else \
        np.all((p[:, :2] > lo[:2] + 1e-9) & (p[:, :2] < hi[:2] - 1e-9), axis=1)
    rng = np.random.default_rng(seed)
    d = rng.uniform(-amplitude, amplitude, p.shape)
    if keep_z:
        d[:, 2] = 0.0
    p[inner] += d[inner]
    return p
