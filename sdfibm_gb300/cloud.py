"""Python mirror of sdfibm's SolidCloud API (src/solidcloud.h:89-124) on the GB300 coupling library.

    cloud = SolidCloud(mesh, solids, options)          # SolidCloud::SolidCloud after solidDict parsing
    FT = cloud.interact(t, dt, U, fields)              # SolidCloud::interact   (fields: As, Fs, Ts, Ct)
    cloud.evolve(t, dt)                                # SolidCloud::evolve
    cloud.fix_internal(fields["Ct"], U)                # SolidCloud::fixInternal
    cloud.states() / cloud.set_states(st)              # Solid getters / setters
    cloud.save_state(state_file, U, Ct)                # SolidCloud::saveState   (state_file: host.StateFile)
    cloud.set_sampler(shape); cloud.mean_field(U, Ct)  # meta.sampler, SolidCloud::calcMeanField
    cloud.initial_correct(U, fields), cloud.total_solid_volume(fields), cloud[i], cloud.is_on_twod()
    cloud.save_restart(dict_text, path)                # SolidCloud::saveRestart

Fields are CUDA tensors in the cell-major layout of include/sdfibm_cuda.h: U and Fs have shape (3, N) float32,
As and Ts (N,) float32, Ct (N,) int32.  Every call goes through libsdfibm_cuda.so; errors raise CouplingError
carrying the library's status and message.
"""
import ctypes as C

import numpy as np

from . import abi
from . import host
from ._lib import load


class CouplingError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("sdfibm_cuda status %d: %s" % (status, msg))
        self.status = status


def _ptr(t):
    return C.c_void_p(t.data_ptr())


class SolidCloud:
    def __init__(self, mesh, solids, opt=None, stream=None, time=0.0):
        self._L = load()
        self.mesh = mesh
        self.time = float(time)  # m_time: the construction time, then the time of the last evolve
        self._stream = stream
        self._sampler = None     # (shape, SolidCloud of the solids with that shape) for mean_field
        self._sampler_fields = None
        self._sampler_ct = None  # (Ct written by mean_field, mask of its cells), zeroed before the next interact
        self.nsolids = len(solids)
        self.ncells = int(mesh.nx) * int(mesh.ny) * int(mesh.nz)
        self._solids = (abi.SolidDesc * max(1, len(solids)))(*solids)
        self.opt = opt if opt is not None else abi.options()
        self._h = C.c_void_p()
        s = C.c_void_p(stream.cuda_stream) if stream is not None else None
        rc = self._L.sdfibm_cuda_create(C.byref(mesh), self._solids, len(solids), C.byref(self.opt), s,
                                        C.byref(self._h))
        if rc != abi.OK:
            raise CouplingError(rc, "create failed")

    @classmethod
    def from_polymesh(cls, points, face_off, face_lab, owner, neighbour, solids, opt=None, twod=False, stream=None):
        """SolidCloud on an explicit OpenFOAM polyMesh (graded, multi-block or polyhedral): the polyMesh lists as
        read from constant/polyMesh (points [P, 3], faces as offsets [F + 1] and labels, owner [F], neighbour [F_int]).
        The reference's REF-GEO fraction; fields are cell-major as for the uniform mesh, ncells = max label + 1."""
        self = cls.__new__(cls)
        self._L = load()
        self.mesh = None
        self.time = 0.0
        self._stream = stream
        self._sampler = None
        self._sampler_fields = None
        self._sampler_ct = None
        self.nsolids = len(solids)
        self._solids = (abi.SolidDesc * max(1, len(solids)))(*solids)
        self.opt = opt if opt is not None else abi.options()
        self._poly = tuple(np.ascontiguousarray(a, dt) for a, dt in ((points, np.float64), (face_off, np.int32),
                                                                     (face_lab, np.int32), (owner, np.int32),
                                                                     (neighbour, np.int32)))
        pts, fo, fl, ow, nb = self._poly
        self.ncells = int(max(ow.max(initial=-1), nb.max(initial=-1))) + 1
        self._h = C.c_void_p()
        s = C.c_void_p(stream.cuda_stream) if stream is not None else None
        p = lambda a: a.ctypes.data_as(C.c_void_p)
        rc = self._L.sdfibm_cuda_create_polymesh(p(pts), len(pts), p(fo), p(fl), len(fo) - 1, p(ow), p(nb), len(nb),
                                                 int(bool(twod)), self._solids, len(solids), C.byref(self.opt), s,
                                                 C.byref(self._h))
        if rc != abi.OK:
            raise CouplingError(rc, "polyMesh create failed")
        return self

    def _check(self, rc):
        if rc != abi.OK:
            raise CouplingError(rc, self._L.sdfibm_cuda_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_sampler", None) is not None:
            self._sampler[1].close()
            self._sampler = None
            self._sampler_fields = None
        if getattr(self, "_h", None) and self._h.value:
            self._L.sdfibm_cuda_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def new_fields(self, device="cuda"):
        import torch
        N = self.ncells
        return dict(As=torch.zeros(N, dtype=torch.float32, device=device),
                    Fs=torch.zeros(3, N, dtype=torch.float32, device=device),
                    Ts=torch.zeros(N, dtype=torch.float32, device=device),
                    Ct=torch.zeros(N, dtype=torch.int32, device=device))

    def interact(self, time, dt, U, fields, want_ft=True):
        self._clear_sampler_ct(fields["Ct"])
        FT = np.zeros((max(1, self.nsolids), 6)) if want_ft else None
        rc = self._L.sdfibm_cuda_interact(self._h, float(time), float(dt), _ptr(U), _ptr(fields["As"]),
                                          _ptr(fields["Fs"]), _ptr(fields["Ts"]), _ptr(fields["Ct"]),
                                          FT.ctypes.data_as(C.c_void_p) if want_ft else None)
        self._check(rc)
        return FT[:self.nsolids] if want_ft else None

    def interact_host(self, time, dt, U, fields):
        """Host (numpy) fields.  Page-locked field arrays (e.g. numpy views of torch pin_memory tensors) receive only
        the cells that changed since the previous call on the same arrays, written in place; other arrays receive
        whole-field copies."""
        FT = np.zeros((max(1, self.nsolids), 6))
        p = lambda a: a.ctypes.data_as(C.c_void_p)
        rc = self._L.sdfibm_cuda_interact_host(self._h, float(time), float(dt), p(U), p(fields["As"]), p(fields["Fs"]),
                                               p(fields["Ts"]), p(fields["Ct"]), p(FT))
        self._check(rc)
        return FT[:self.nsolids]

    def interact_host64(self, time, dt, U, fields):
        """FP64 host (numpy) fields in OpenFOAM's layout: U and Fs [N, 3], As, Ts, Ct [N] (Ct as float64).
        Page-locked arrays are read and written in place by the GPU; other arrays are staged through whole-field
        copies."""
        FT = np.zeros((max(1, self.nsolids), 6))
        for k, a in (("U", U),) + tuple(fields.items()):
            if a.dtype != np.float64 or not a.flags.c_contiguous:
                raise ValueError("interact_host64: %s must be a C-contiguous float64 array" % k)
        p = lambda a: a.ctypes.data_as(C.c_void_p)
        rc = self._L.sdfibm_cuda_interact_host64(self._h, float(time), float(dt), p(U), p(fields["As"]),
                                                 p(fields["Fs"]), p(fields["Ts"]), p(fields["Ct"]), p(FT))
        self._check(rc)
        return FT[:self.nsolids]

    def initial_correct(self, U, fields):
        """SolidCloud::initialCorrect (src/solidcloud.cpp:276-286): interact(0, 1), then every solid's force and
        torque cleared (the fluid force of that pass stays, as in the reference).  Returns the per-solid force and
        torque of the pass."""
        FT = self.interact(0.0, 1.0, U, fields)
        st = self.states()
        for x in st:
            for a in range(3):
                x.force[a] = 0.0
                x.torque[a] = 0.0
        self.set_states(st)
        return FT

    def total_solid_volume(self, fields):
        """SolidCloud::totalSolidVolume (src/solidcloud.cpp:572-576): sum of As times the cell volume."""
        V = float(self.mesh.h[0]) * float(self.mesh.h[1]) * float(self.mesh.h[2])
        return float(fields["As"].double().sum()) * V

    def is_on_fluid(self):
        """SolidCloud::isOnFluid: meta.on_fluid (a cloud without fluid coupling has rho_f = 0)."""
        return self.opt.rho_f != 0.0

    def is_on_twod(self):
        """SolidCloud::isOnTwoD: meta.on_twod."""
        return bool(self.mesh.twod)

    def __getitem__(self, i):
        """SolidCloud::operator[] (src/solidcloud.cpp:667-670): the state of solid i."""
        if not 0 <= i < self.nsolids:
            raise IndexError(i)
        return self.states()[i]

    def __len__(self):
        return self.nsolids

    def evolve(self, time, dt):
        self._check(self._L.sdfibm_cuda_evolve(self._h, float(time), float(dt)))
        self.time = float(time)

    def fix_internal(self, Ct, U):
        self._check(self._L.sdfibm_cuda_fix_internal(self._h, _ptr(Ct), _ptr(U)))

    def apply_forcing(self, dt, fields, U, T=None):
        """The solver's forcing update on device fields (main.cpp:70-77): U -= Fs dt, T = (1 - As) T + Ts, from the
        fields the last interact wrote (sdfibm_cuda_apply_forcing)."""
        self._check(self._L.sdfibm_cuda_apply_forcing(self._h, float(dt), _ptr(fields["As"]), _ptr(fields["Fs"]),
                                                       _ptr(fields["Ts"]), _ptr(U),
                                                       _ptr(T) if T is not None else None))

    def states(self):
        st = (abi.SolidState * max(1, self.nsolids))()
        self._check(self._L.sdfibm_cuda_get_solids(self._h, st, self.nsolids))
        return list(st)[:self.nsolids]

    def set_states(self, states):
        arr = (abi.SolidState * max(1, self.nsolids))(*states)
        self._check(self._L.sdfibm_cuda_set_solids(self._h, arr, self.nsolids))

    def set_sampler(self, shape):
        """meta.sampler: the shape (a host.make_shape descriptor) that mean_field puts on every solid."""
        if self._sampler is not None:
            self._sampler[1].close()
            self._sampler_fields = None
        solids = []
        for d in self._solids[:self.nsolids]:
            e = abi.SolidDesc.from_buffer_copy(d)
            e.shape = shape
            solids.append(e)
        # at rest, rho_f = 1, FP64 forcing, the reference's REF-GEO fraction (calcMeanField calls calcCellVolume)
        opt = abi.options(rho_f=1.0, fraction_method=abi.FRACTION_REFGEO, exact_forcing=1)
        self._sampler = (shape, SolidCloud(self.mesh, solids, opt, stream=self._stream))

    def mean_field(self, U, Ct=None):
        """SolidCloud::calcMeanField (src/solidcloud.cpp:315-359) of U for every solid, with the sampler shape in
        the solid's pose: sum(alpha V U) / sum(alpha V) over the cells the sampler touches, alpha the REF-GEO fraction
        (1 inside).  Returns (S, 3) float64.

        Computed by the coupling itself: the sampler-shaped solids at rest, with rho_f = 1 and dt = 1, receive the
        force sum(alpha V (U - 0)); a second pass on U = 1 gives sum(alpha V).  Like the reference (writeMeanField
        runs before fixInternal), Ct, when given, is overwritten on every cell a sampler touches: id + 4 inside, the
        cell type on cut cells."""
        if self._sampler is None:
            raise CouplingError(5, "mean_field needs a sampler shape (set_sampler)")
        import torch
        sc = self._sampler[1]
        st = self.states()
        for x in st:
            for a in range(3):
                x.vel[a] = 0.0
                x.omega[a] = 0.0
        sc.set_states(st)
        if self._sampler_fields is None or self._sampler_fields["As"].device != U.device:
            self._sampler_fields = sc.new_fields(device=U.device)
        f = self._sampler_fields
        F = sc.interact(self.time, 1.0, U, f)
        W = sc.interact(self.time, 1.0, torch.ones_like(U), f)
        if Ct is not None:
            sct = f["Ct"]
            Ct.copy_(torch.where(sct != 0, sct, Ct))
            # the reference's next interact zeroes every cell (solidcloud.cpp:438-441); the sparse reset covers the
            # coupling's own cells, so the sampler's are remembered and zeroed before that call
            self._sampler_ct = (Ct, sct != 0)
        return F[:, :3] / W[:, :1]

    def _clear_sampler_ct(self, Ct):
        mark = getattr(self, "_sampler_ct", None)
        if mark is not None and mark[0].data_ptr() == Ct.data_ptr():
            Ct.masked_fill_(mark[1], 0)
        self._sampler_ct = None

    def save_state(self, state_file, U=None, Ct=None):
        """SolidCloud::saveState: appends this step's records to a host.StateFile (cloud.out) and, when the file
        keeps the mean field and a sampler is set, the mean of U around every solid (meanfield.out)."""
        mf = None
        if state_file.keeps_mean_field and self._sampler is not None:
            if U is None:
                raise CouplingError(1, "the mean field needs U")
            mf = self.mean_field(U, Ct)
        state_file.save(self.time, self.states(), mf)

    def save_restart(self, dict_text, path, precision=6, stamp=None):
        """SolidCloud::saveRestart: writes the solidDict read at construction (dict_text) with every solid's pos,
        vel, euler and omega set to its current state."""
        text = host.write_restart(dict_text, self.states(), bool(self.mesh.twod), precision, stamp)
        with open(path, "w") as f:
            f.write(text)

    def touched(self, s):
        n = C.c_int64(0)
        self._check(self._L.sdfibm_cuda_touched(self._h, int(s), None, None, 0, C.byref(n)))
        cells = np.zeros(max(1, n.value), np.int64)
        types = np.zeros(max(1, n.value), np.int8)
        self._check(self._L.sdfibm_cuda_touched(self._h, int(s), cells.ctypes.data_as(C.c_void_p),
                                                types.ctypes.data_as(C.c_void_p), n.value, C.byref(n)))
        return cells[:n.value], types[:n.value]

    def kernel_times(self):
        """{kernel name: device ms} of the last interact (options.timing must be set)."""
        names = (C.c_char_p * 32)()
        ms = (C.c_double * 32)()
        n = C.c_int32(0)
        self._check(self._L.sdfibm_cuda_kernel_times(self._h, names, ms, 32, C.byref(n)))
        out = {}
        for i in range(n.value):
            k = names[i].decode()
            out[k] = out.get(k, 0.0) + ms[i]
        return out

    def stats(self):
        out = (C.c_int64 * 11)()
        self._check(self._L.sdfibm_cuda_stats(self._h, out, 11))
        keys = ("coupling_cells", "cut_cells", "bbox_cells", "fp64_rechecks", "work_items", "launches",
                "learned_cells", "learned_fallback_cells", "host_h2d_bytes", "host_d2h_bytes", "host_sparse")
        return dict(zip(keys, list(out)))

    def autotune(self, dt, U, fields):
        """Chooses the launch configuration (classify work-item size, CTA counts) by timing dense interacts on these
        fields (or takes it from the per-shape cache); returns tiles per item."""
        out = C.c_int32(0)
        self._check(self._L.sdfibm_cuda_autotune(self._h, float(dt), _ptr(U), _ptr(fields["As"]), _ptr(fields["Fs"]),
                                                 _ptr(fields["Ts"]), _ptr(fields["Ct"]), C.byref(out)))
        return out.value

    def tuning(self):
        """The launch configuration in use (what the autotuner chose, or the defaults)."""
        out = (C.c_int32 * 7)()
        self._check(self._L.sdfibm_cuda_tuning(self._h, out, 7))
        keys = ("classify_tiles_per_item", "classify_ctas", "subsample_ctas", "couple_ctas", "mlp_ctas",
                "refgeo_ctas", "from_cache")
        return dict(zip(keys, list(out)))

    def set_fraction_model(self, params, tau_refine, rho_min):
        """Installs the learned cut-cell fraction model (options.fraction_method = FRACTION_LEARNED) and its band:
        cells whose planar reconstructions disagree by more than tau_refine, or whose solid's bounding radius spans
        fewer than rho_min cells, take the SUBSAMPLE fallback."""
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.shape != (abi.MLP_NPARAM,):
            raise ValueError("fraction model needs %d parameters" % abi.MLP_NPARAM)
        self._check(self._L.sdfibm_cuda_set_fraction_model(self._h, p.ctypes.data_as(C.c_void_p),
                                                           C.c_float(tau_refine), C.c_float(rho_min)))
