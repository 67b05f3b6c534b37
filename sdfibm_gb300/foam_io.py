"""OpenFOAM file input and field output through the host half of libsdfibm_cuda.so (include/sdfibm_host.h): the
lists of polyMesh files and field internalFields, ascii or binary, vol field files with a new internalField, and the
uniform mesh a single-block polyMesh describes.

    read_list(path, "vector")            points (N, 3); "label" for owner / neighbour; "scalar" for scalar fields
    read_faces(path)                     (offsets, labels) of a faceCompactList or faceList
    write_field(template, values)        a vol field file with its internalField set (scalars or vectors)
    uniform_mesh_from_polymesh(dir)      abi.MeshDesc of constant/polyMesh when it is one uniform block
"""
import ctypes as C
import os

import numpy as np

from . import abi
from ._lib import load
from .host import HostError

_KINDS = {"scalar": (0, np.float64, 1), "vector": (1, np.float64, 3), "label": (2, np.int32, 1)}


def _bytes(path_or_bytes):
    if isinstance(path_or_bytes, (bytes, bytearray)):
        return bytes(path_or_bytes)
    with open(path_or_bytes, "rb") as f:
        return f.read()


def read_list(path_or_bytes, kind):
    """The list of an OpenFOAM file as a numpy array; for a uniform vol*Field the single value (shape (1,) or (1, 3))
    with uniform=True in a tuple (array, True), else (array, False)."""
    data = _bytes(path_or_bytes)
    k, dt, width = _KINDS[kind]
    L = load()
    n = C.c_int64(0)
    msg = C.create_string_buffer(512)
    if L.sdfibm_host_read_foam_list(data, len(data), k, None, 0, C.byref(n), msg, 512) != abi.OK:
        raise HostError(msg.value.decode())
    uniform = n.value < 0
    m = 1 if uniform else n.value
    out = np.zeros((m, width) if width > 1 else m, dtype=dt)
    if L.sdfibm_host_read_foam_list(data, len(data), k, out.ctypes.data_as(C.c_void_p), m, C.byref(n), msg,
                                    512) != abi.OK:
        raise HostError(msg.value.decode())
    return out, uniform


def read_faces(path_or_bytes):
    """(offsets (nfaces + 1,), labels) of a polyMesh faces file."""
    data = _bytes(path_or_bytes)
    L = load()
    nf, nl = C.c_int64(0), C.c_int64(0)
    msg = C.create_string_buffer(512)
    if L.sdfibm_host_read_foam_faces(data, len(data), None, 0, None, 0, C.byref(nf), C.byref(nl), msg, 512) != abi.OK:
        raise HostError(msg.value.decode())
    off = np.zeros(nf.value + 1, np.int32)
    lab = np.zeros(max(1, nl.value), np.int32)
    if L.sdfibm_host_read_foam_faces(data, len(data), off.ctypes.data_as(C.c_void_p), len(off),
                                     lab.ctypes.data_as(C.c_void_p), len(lab), C.byref(nf), C.byref(nl), msg,
                                     512) != abi.OK:
        raise HostError(msg.value.decode())
    return off, lab[:nl.value]


def write_field(template, values, fmt=None, precision=6):
    """The bytes of an OpenFOAM vol field file: template (bytes of a volScalarField or volVectorField file) with its
    internalField set to values, (N,) scalars or (N, 3) vectors (a cell-major (3, N) field is transposed first).
    fmt: None keeps the template's format, else "ascii" or "binary"."""
    v = np.asarray(values, dtype=np.float64)
    if v.ndim == 2 and v.shape[0] == 3 and v.shape[1] != 3:
        v = v.T
    vector = v.ndim == 2
    v = np.ascontiguousarray(v)
    f = {None: -1, "ascii": 0, "binary": 1}[fmt]
    L = load()
    fn = L.sdfibm_host_write_vector_field if vector else L.sdfibm_host_write_scalar_field
    n = C.c_int64(0)
    msg = C.create_string_buffer(512)
    args = (template, len(template), v.ctypes.data_as(C.c_void_p), len(v), f, int(precision))
    if fn(*args, None, 0, C.byref(n), msg, 512) != abi.OK:
        raise HostError(msg.value.decode())
    buf = C.create_string_buffer(n.value + 1)
    if fn(*args, buf, n.value + 1, C.byref(n), msg, 512) != abi.OK:
        raise HostError(msg.value.decode())
    return buf.raw[:n.value]


def uniform_mesh(points, ncells, rtol=1e-9):
    """abi.MeshDesc of a single-block point lattice (x fastest, then y, then z)."""
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    m = abi.MeshDesc()
    msg = C.create_string_buffer(512)
    if load().sdfibm_host_uniform_mesh(pts.ctypes.data_as(C.c_void_p), len(pts), int(ncells), float(rtol), C.byref(m),
                                       msg, 512) != abi.OK:
        raise HostError(msg.value.decode())
    return m


def uniform_mesh_from_polymesh(polymesh_dir, rtol=1e-9):
    """The uniform mesh of a polyMesh directory (points, owner): its cell count is the largest owner label + 1."""
    pts, _ = read_list(os.path.join(polymesh_dir, "points"), "vector")
    own, _ = read_list(os.path.join(polymesh_dir, "owner"), "label")
    return uniform_mesh(pts, int(own.max()) + 1 if len(own) else 0, rtol)
