"""The VOF initializer of sdfibm (tool_vof/main.cpp, SolidCloud::writeVOF tool_vof/solidcloud.cpp:117-173) on the
GB300 coupling library: a smooth phase field, the solids' volume fraction per cell, for a two-phase case.

    python -m sdfibm_gb300.vof [CASE] [--name alpha.water] [--no-planes]

reads CASE/solidDict (the tool's format: meta.on_twod, shapes, solids and planes with pos / euler / shp_name),
the single uniform block of CASE/system/blockMeshDict (or constant/polyMesh/blockMeshDict, or the polyMesh itself
when it is one uniform block) and CASE/0/<name>, and
writes CASE/0/<name> with its internalField set to the field, in the case's writeFormat and writePrecision.

The field is one coupling pass on the GPU: sdfibm_cuda_interact of the solids at rest with the REF-GEO fraction
leaves As = min(sum of the fractions, 1), the value writeVOF accumulates with a clamp after every solid.  There is
no CPU path: without libsdfibm_cuda.so or a GPU the call fails.
"""
import argparse
import ctypes as C
import os
import sys

import numpy as np

from . import abi
from ._lib import load
from .host import HostError, soliddict_lookup


def parse_vofdict(text, with_planes=True):
    """tool_vof's solidDict: returns (solids, on_twod)."""
    L = load()
    n, tw = C.c_int32(0), C.c_int32(0)
    msg = C.create_string_buffer(512)
    rc = L.sdfibm_host_parse_vofdict(text.encode(), int(bool(with_planes)), None, 0, C.byref(n), C.byref(tw), msg, 512)
    if rc != abi.OK and n.value == 0:
        raise HostError(msg.value.decode())
    arr = (abi.SolidDesc * max(1, n.value))()
    rc = L.sdfibm_host_parse_vofdict(text.encode(), int(bool(with_planes)), arr, n.value, C.byref(n), C.byref(tw),
                                     msg, 512)
    if rc != abi.OK:
        raise HostError(msg.value.decode())
    return list(arr)[:n.value], bool(tw.value)


def parse_blockmesh(text):
    """The uniform mesh of a one-block blockMeshDict (abi.MeshDesc)."""
    m = abi.MeshDesc()
    msg = C.create_string_buffer(512)
    if load().sdfibm_host_parse_blockmesh(text.encode(), C.byref(m), msg, 512) != abi.OK:
        raise HostError(msg.value.decode())
    return m


def write_scalar_field(template, values, fmt=None, precision=6):
    """The bytes of an OpenFOAM volScalarField file: template (bytes) with its internalField set to values.
    fmt: None keeps the template's format, else "ascii" or "binary"."""
    v = np.ascontiguousarray(values, dtype=np.float64).reshape(-1)
    f = {None: -1, "ascii": 0, "binary": 1}[fmt]
    L = load()
    n = C.c_int64(0)
    msg = C.create_string_buffer(512)
    args = (template, len(template), v.ctypes.data_as(C.c_void_p), len(v), f, int(precision))
    if L.sdfibm_host_write_scalar_field(*args, None, 0, C.byref(n), msg, 512) != abi.OK:
        raise HostError(msg.value.decode())
    buf = C.create_string_buffer(n.value + 1)
    if L.sdfibm_host_write_scalar_field(*args, buf, n.value + 1, C.byref(n), msg, 512) != abi.OK:
        raise HostError(msg.value.decode())
    return buf.raw[:n.value]


def smooth_vof(mesh, solids, device="cuda"):
    """The phase field (N,) float64 of the solids on the mesh: As of one REF-GEO coupling pass at rest."""
    import torch
    from .cloud import SolidCloud
    opt = abi.options(rho_f=1.0, fraction_method=abi.FRACTION_REFGEO)
    cloud = SolidCloud(mesh, solids, opt)
    try:
        f = cloud.new_fields(device=device)
        U = torch.zeros((3, cloud.ncells), dtype=torch.float32, device=device)
        cloud.interact(0.0, 1.0, U, f, want_ft=False)
        return f["As"].double().cpu().numpy()
    finally:
        cloud.close()


def _read(path, mode="r"):
    with open(path, mode) as fh:
        return fh.read()


def run_case(case, name="alpha.water", with_planes=True, log=print):
    """tool_vof's main: writes CASE/0/<name>; returns the field."""
    solids, twod = parse_vofdict(_read(os.path.join(case, "solidDict")), with_planes)
    pm = os.path.join(case, "constant", "polyMesh")
    for sub in ("system", os.path.join("constant", "polyMesh")):
        bm = os.path.join(case, sub, "blockMeshDict")
        if os.path.exists(bm):
            mesh = parse_blockmesh(_read(bm))
            break
    else:
        if not os.path.exists(os.path.join(pm, "points")):
            raise HostError("no blockMeshDict and no polyMesh in %s" % case)
        from .foam_io import uniform_mesh_from_polymesh
        mesh = uniform_mesh_from_polymesh(pm)  # a single uniform block, or HostError
    mesh.twod = int(twod)
    ctrl = _read(os.path.join(case, "system", "controlDict"))
    fmt = soliddict_lookup(ctrl, "writeFormat", "ascii")
    prec = int(soliddict_lookup(ctrl, "writePrecision", "6"))
    field_path = os.path.join(case, "0", name)
    template = _read(field_path, "rb")
    alpha = smooth_vof(mesh, solids)
    for c in np.flatnonzero((alpha < 0) | (alpha > 1 + 1e-6)):
        log("Wrong volume fraction %g at cell %d" % (alpha[c], c))
    with open(field_path, "wb") as fh:
        fh.write(write_scalar_field(template, alpha, fmt if fmt in ("ascii", "binary") else None, prec))
    vol = float((alpha * (mesh.h[0] * mesh.h[1] * mesh.h[2])).sum())
    log("* Write smooth phase field [%s] to ./0, total volume = %.6g" % (name, vol))
    return alpha


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("case", nargs="?", default=".")
    ap.add_argument("--name", default="alpha.water", help="name of the field to initialise")
    ap.add_argument("--no-planes", action="store_true", help="ignore the solidDict's planes entries")
    a = ap.parse_args(argv)
    run_case(a.case, a.name, not a.no_planes)
    return 0


if __name__ == "__main__":
    sys.exit(main())
