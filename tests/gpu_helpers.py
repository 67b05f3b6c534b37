"""Shared helpers of the GPU parity tests: run one workload through libsdfibm_cuda.so and through the oracle."""
import numpy as np

from oracle.oracle import OracleCloud
from sdfibm_gb300 import abi
from sdfibm_gb300.cloud import SolidCloud

# tolerances (stated by the coupling contract)
AS_REL, AS_ABS = 1e-5, 1e-9      # As, Ts and Fs per cell: |d| <= 1e-5 |ref| + 1e-9
FT_REL = 1e-6                    # force/torque per solid, normwise against the sum of |contributions|


def run_pair(torch, w, steps=1, evolve=False, fix=False, U=None, gpu_opt=None, gpu_setup=None, sync_states=False):
    """Runs `steps` interact (+evolve, +fixInternal) on the GPU and on the fast oracle; returns both sides.

    gpu_opt: options of the GPU side when they differ from the oracle's (w.opt); gpu_setup(cloud) runs after
    the GPU cloud is created.  sync_states: the oracle takes the GPU's solid states before every interact, so that
    each step compares the coupling on the same states (the FP32 forcing's force sums, within their 1e-6 bound, move
    the solids by a little through evolve, and U - us can cancel at a cell)."""
    Uh = w.U_numpy() if U is None else U
    gpu = SolidCloud(w.mesh, w.solids, gpu_opt if gpu_opt is not None else w.opt)
    if gpu_setup is not None:
        gpu_setup(gpu)
    orc = OracleCloud(w.mesh, w.solids, w.opt, faithful=False)
    Ud = torch.from_numpy(Uh).cuda()
    Uo = Uh.astype(np.float64).reshape(-1).copy()
    fd = gpu.new_fields()
    fo = orc.new_fields()
    out = []
    t = 0.0
    for _ in range(steps):
        if sync_states:
            orc.set_state(gpu.states())
        FTg = gpu.interact(t, w.dt, Ud, fd)
        FTo = orc.interact(t, w.dt, Uo, fo)
        out.append((FTg, FTo))
        if evolve:
            gpu.evolve(t, w.dt)
            orc.evolve(t, w.dt)
        if fix:
            gpu.fix_internal(fd["Ct"], Ud)
            Uo = orc.fix_internal(fo["Ct"], Uo)
        t += w.dt
    torch.cuda.synchronize()
    return dict(gpu=gpu, orc=orc, fd=fd, fo=fo, FT=out, Ud=Ud, Uo=Uo)


def centres(m, cells):
    """Cell centres [3, n] of cell labels (numpy)."""
    cells = np.asarray(cells, dtype=np.int64)
    i = cells % m.nx
    j = (cells // m.nx) % m.ny
    k = cells // (m.nx * m.ny)
    return np.stack([m.origin[0] + (i + 0.5) * m.h[0], m.origin[1] + (j + 0.5) * m.h[1],
                     m.origin[2] + (k + 0.5) * m.h[2]])


def ft_scale(w, orc, fo_U, s, cells=None, st=None):
    """rho_f * V/dt * sum over the solid's cells of |U - u_s| (and of |C-x| |U - u_s| for the torque)."""
    if cells is None:
        cells, _ = orc.touched(s)
    N = orc.N
    U = fo_U.reshape(3, N)[:, cells]
    st = (st if st is not None else orc.get_state())[s]
    C = centres(w.mesh, cells)
    x = np.array(st.pos)[:, None]
    v = np.array(st.vel)[:, None]
    om = np.array(st.omega)
    d = C - x
    us = v + np.cross(om, d.T).T
    fm = np.linalg.norm(U - us, axis=0) * 1.5  # alpha <= ~1.5 for REF-GEO cut cells
    V = w.mesh.h[0] * w.mesh.h[1] * w.mesh.h[2]
    k = w.opt.rho_f * V / w.dt
    return k * fm.sum() + 1e-300, k * (np.linalg.norm(d, axis=0) * fm).sum() + 1e-300


def _centre(m, c):
    return tuple(centres(m, [c])[:, 0])


def check_interact(w, r, U_used=None):
    """Asserts the coupling contract on the last interact of run_pair; returns a summary dict."""
    gpu, orc, fd, fo = r["gpu"], r["orc"], r["fd"], r["fo"]
    N = orc.N
    S = len(w.solids)
    ncells = 0
    for s in range(S):
        cg, tg = gpu.touched(s)
        co, to = orc.touched(s)
        assert np.array_equal(cg, co), "touched cells of solid %d differ (%d vs %d)" % (s, len(cg), len(co))
        assert np.array_equal(tg, to), "cell types of solid %d differ" % s
        ncells += len(co)
    Ct = fd["Ct"].cpu().numpy()
    assert np.array_equal(Ct, fo["Ct"]), "Ct differs in %d cells" % int((Ct != fo["Ct"]).sum())
    for key in ("As", "Ts"):
        g = fd[key].cpu().numpy().astype(np.float64)
        o = fo[key]
        bad = np.abs(g - o) > AS_REL * np.abs(o) + AS_ABS
        assert not bad.any(), "%s differs in %d cells, worst %g vs %g" % (key, bad.sum(), g[bad][0], o[bad][0])
    g = fd["Fs"].cpu().numpy().astype(np.float64).reshape(3, N)
    o = fo["Fs"].reshape(3, N)
    # Fs is relative-accurate per contribution; where several solids touch one cell their contributions can cancel,
    # so there the bound is taken against the sum of the contributions' magnitudes
    scale = np.abs(o).copy()
    touched = [orc.touched(s)[0] for s in range(S)]
    allc = np.concatenate(touched) if S else np.zeros(0, np.int64)
    alls = np.concatenate([np.full(len(t), s) for s, t in enumerate(touched)]) if S else np.zeros(0, np.int64)
    uc, cnt = np.unique(allc, return_counts=True)
    shared = set(uc[cnt > 1].tolist())
    owners = {}
    if shared:
        for c, s in zip(allc.tolist(), alls.tolist()):
            if c in shared:
                owners.setdefault(c, []).append(s)
    Uo = r["Uo"].reshape(3, N) if U_used is None else U_used.reshape(3, N)
    st = orc.get_state()
    for c, ss in owners.items():
        C = np.array(_centre(w.mesh, c))
        mag = np.zeros(3)
        for s in ss:
            al = orc.cell_fraction(s, c, int(w.opt.fraction_method))  # the solid's own fraction of the cell
            x = np.array(st[s].pos)
            us = np.array(st[s].vel) + np.cross(np.array(st[s].omega), C - x)
            mag += al * np.abs(Uo[:, c] - us) / w.dt
        scale[:, c] = np.maximum(scale[:, c], mag)
    bad = np.abs(g - o) > AS_REL * scale + AS_ABS
    assert not bad.any(), "Fs differs in %d entries" % bad.sum()
    FTg, FTo = r["FT"][-1]
    Uo = r["Uo"] if U_used is None else U_used
    worst = 0.0
    states = orc.get_state()
    for s in range(S):
        sf, st = ft_scale(w, orc, Uo, s, cells=touched[s], st=states)
        ef = np.linalg.norm(FTg[s, :3] - FTo[s, :3]) / sf
        et = np.linalg.norm(FTg[s, 3:] - FTo[s, 3:]) / st
        worst = max(worst, ef, et)
        assert ef <= FT_REL and et <= FT_REL, "solid %d force/torque error %g %g" % (s, ef, et)
    return dict(coupling_cells=ncells, ft_err=worst)
