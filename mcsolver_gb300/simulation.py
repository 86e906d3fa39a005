"""mcsolver parameter files and the (T, H) grid driver on the engine.

The reference drives its compiled libraries from a version-3.0 parameter file
(fileio.loadParam, fileio.py:169-313): lattice vectors, supercell, orbitals
(spin length, position, single-ion anisotropy), bonds (3x3 exchange matrices),
the temperature and field grids, the correlated orbital pair, orbital groups,
local circuits, sweep counts, model and algorithm.  win.startSimulation
(win.py:40-180) fans the grid out over a process pool, one MCMainFunction call
per (T, H) point, and mcMain writes ``out``, ``spinDotSpin.txt``, spin frames
and ``result.txt`` (mcMain.py:126-135, :259-289, :291-323; win.py:170-177).

Here the whole grid is one batch on the GPU: every point becomes one replica of
``mcsolver_gb300.Batch`` (the tuples are built with the reference's site order
and couplings divided by the clamped temperature; the lattice is built once by
``lattice.LatticeTemplate`` and each point rescales J, D and h), and
the same files are written with the reference's formats, points in grid order
(H outer, T inner; the reference writes them in pool completion order).

Differences on purpose: the bond objects are not renormalised in place
(Lattice.py:141-147 divides each bond's strength by T on every use); a dipole
term (alpha != 0) is rejected, since the reference's dipole path fails
(Lattice.py:298 calls addLinking without its distance argument).
"""
from __future__ import annotations

import os
import re
from concurrent.futures import ThreadPoolExecutor

import numpy as np

SETTING_FILE_VERSION = "3.0"
_TAGS = ("Lattice", "Supercell", "Orbitals", "Bonds", "Temperature", "Field", "Dipole", "Sweeps", "Model",
         "Algorithm", "Measurement", "OrbGroup", "Ncores", "Distribution", "XAxis", "LocalCircuit")


def _nums(pattern, line):
    return re.findall(pattern, line)


def load_param(path: str) -> dict:
    """Parse a version-3.0 parameter file the way fileio.loadParam does
    (fileio.py:169-313): tags are the first word of a line (the last line
    carrying a tag wins), numbers are read from the lines after each tag.
    Raises ValueError on an unknown version or a missing tag."""
    with open(path) as f:
        data = [line for line in f.read().split("\n") if line]
    if not data:
        raise ValueError("empty parameter file")
    v = _nums(r"[0-9\.]+", data[0])
    if not v or v[0] != SETTING_FILE_VERSION:
        raise ValueError("unknown file or version (only version %s is read)" % SETTING_FILE_VERSION)
    tag = {}
    for i, line in enumerate(data):
        kw = _nums(r"[a-zA-Z]+", line)
        if kw and kw[0] in _TAGS:
            tag[kw[0]] = i
    missing = [t for t in _TAGS if not tag.get(t)]
    if missing:
        raise ValueError("cannot find some tags: " + ", ".join(missing))
    p = {}
    p["LMatrix"] = [[float(x) for x in _nums(r"[0-9\.\-]+", data[tag["Lattice"] + 1 + i])] for i in range(3)]
    p["LPack"] = [int(x) for x in _nums(r"[0-9]+", data[tag["Supercell"] + 1])]
    norb = int(_nums(r"[0-9]+", data[tag["Orbitals"] + 1])[0])
    p["pos"], p["S"], p["DList"] = [], [], []
    for i in range(norb):
        e = _nums(r"[0-9\.\-]+", data[tag["Orbitals"] + 3 + i])
        p["pos"].append([float(e[3]), float(e[4]), float(e[5])])
        p["S"].append(float(e[2]))
        p["DList"].append([float(e[6]), float(e[7]), float(e[8])])
    nb = int(_nums(r"[0-9]+", data[tag["Bonds"] + 1])[0])
    p["bondList"] = []
    for i in range(nb):
        e = _nums(r"[0-9\.\-]+", data[tag["Bonds"] + 3 + i])
        # J in file order Jx Jy Jz Jxy Jxz Jyz Jyx Jzx Jzy = xx yy zz xy xz yz yx zx zy
        p["bondList"].append((int(e[10]), int(e[11]), (int(e[12]), int(e[13]), int(e[14])),
                              [float(x) for x in e[1:10]]))
    s, t, v1, v2, v3 = [int(x) for x in _nums(r"[0-9\-]+", data[tag["Measurement"] + 1])]
    p["GcOrb"] = ((s, t), (v1, v2, v3))
    ng = int(_nums(r"[0-9]+", data[tag["OrbGroup"]])[0])
    p["groupInSC"] = data[tag["OrbGroup"] + 1] == "Supergroup"
    p["orbGroupList"] = []
    for i in range(ng):
        _, o0, o1 = _nums(r"[0-9]+", data[tag["OrbGroup"] + i + 2])
        p["orbGroupList"].append(list(range(int(o0), int(o1) + 1)))
    nc = int(_nums(r"[0-9]+", data[tag["LocalCircuit"]])[0])
    p["localCircuitList"] = []
    for i in range(nc):
        e = [int(x) for x in _nums(r"[0-9\-]+", data[tag["LocalCircuit"] + 1 + i])]
        p["localCircuitList"].append(((e[1], (e[2], e[3], e[4])), (e[5], (e[6], e[7], e[8])), (e[9], (e[10], e[11], e[12]))))
    tp = _nums(r"[0-9\.]+", data[tag["Temperature"] + 1])
    p["T0"], p["T1"], p["nT"] = float(tp[0]), float(tp[1]), int(tp[2])
    hp = _nums(r"[0-9\.\-]+", data[tag["Field"] + 1])
    p["H0"], p["H1"], p["nH"] = float(hp[0]), float(hp[1]), int(hp[2])
    p["dipoleAlpha"] = float(_nums(r"[0-9\.\-]+", data[tag["Dipole"] + 1])[0])
    p["spinFrame"] = int(_nums(r"[0-9]+", data[tag["Distribution"]])[0])
    p["nthermal"], p["nsweep"], p["ninterval"] = [int(x) for x in _nums(r"[0-9\.\-]+", data[tag["Sweeps"] + 1])]
    p["xAxisType"] = data[tag["XAxis"] + 1]
    p["modelType"] = data[tag["Model"] + 1]
    p["algorithm"] = data[tag["Algorithm"] + 1]
    p["ncores"] = int(data[tag["Ncores"] + 1])
    return p


def save_param(p: dict, path: str) -> None:
    """Write a parameter dict in the version-3.0 layout (fileio.saveParam,
    fileio.py:107-167), so that load_param (and the reference) read it back."""
    L = []
    L.append("This is mcsolver's save file, version: 3.0")
    L.append("Lattice:")
    for a in p["LMatrix"]:
        L.append("%.9f %.9f %.9f" % tuple(a))
    L.append("Supercell used in MC simulations:")
    L.append("%d %d %d" % tuple(p["LPack"]))
    L.append("Orbitals in cell:")
    L.append("%d" % len(p["pos"]))
    L.append("Positions, initial spin states and onsite-anisotropy of every orbital:")
    for i, (r, s, d) in enumerate(zip(p["pos"], p["S"], p["DList"])):
        L.append("orb %d: type %d spin %.9f pos [%.9f %.9f %.9f] Dx %.9f Dy %.9f Dz %.9f h %.9f" %
                 (i, i, s, r[0], r[1], r[2], d[0], d[1], d[2], 0.0))
    L.append("Bonds:")
    L.append("%d" % len(p["bondList"]))
    L.append("id, source, target, overLat, exchange matrix elements of each bond:")
    for i, (src, tgt, ov, J) in enumerate(p["bondList"]):
        L.append("bond %d: Jx %.9f Jy %.9f Jz %.9f Jxy %.9f Jxz %.9f Jyz %.9f Jyx %.9f Jzx %.9f Jzy %.9f "
                 "orb %d to orb %d over [%d %d %d]" % ((i,) + tuple(J) + (src, tgt) + tuple(ov)))
    L.append("Temperature scanning region:")
    L.append("Tmin %.9f Tmax %.9f nT %d" % (p["T0"], p["T1"], p["nT"]))
    L.append("Field scanning region (in unit 1.48872 T, only if Kelvin and uB is used for energy and spin):")
    L.append("Hmin %.9f Hmax %.9f nH %d" % (p["H0"], p["H1"], p["nH"]))
    L.append("Dipole long-range coupling:")
    L.append("alpha %.6f" % p.get("dipoleAlpha", 0.0))
    L.append("Measurement:")
    (s, t), ov = p["GcOrb"]
    L.append("measure the correlation function between orb%d and orb%d over [%d %d %d]" % ((s, t) + tuple(ov)))
    L.append("Supergroup")
    L.append("OrbGroup:%d" % len(p.get("orbGroupList", [])))
    L.append("Supergroup" if p.get("groupInSC", True) else "Unitcell")
    for i, g in enumerate(p.get("orbGroupList", [])):
        L.append("group%d orb%d-orb%d" % (i, g[0], g[-1]))
    L.append(">>>       Topological section      <<<")
    L.append("LocalCircuit per cell: %d (set to 0 to skip the calc. for topo. Q)" % len(p.get("localCircuitList", [])))
    for i, c in enumerate(p.get("localCircuitList", [])):
        L.append("Circuit %d enclosed by orb %d [%d %d %d], orb %d [%d %d %d], and orb %d [%d %d %d]" %
                 ((i, c[0][0]) + tuple(c[0][1]) + (c[1][0],) + tuple(c[1][1]) + (c[2][0],) + tuple(c[2][1])))
    L.append(">>>   End of Topological section   <<<")
    L.append("Distribution output frame: %d" % p.get("spinFrame", 0))
    L.append("Sweeps for thermalization and statistics, and relaxiation step for each sweep:")
    L.append("%d %d %d" % (p["nthermal"], p["nsweep"], p["ninterval"]))
    L.append("XAxis type:")
    L.append(p.get("xAxisType", "T"))
    L.append("Model type:")
    L.append(p["modelType"])
    L.append("Algorithm:")
    L.append(p["algorithm"])
    L.append("Ncores:")
    L.append("%d" % p.get("ncores", 1))
    with open(path, "w") as f:
        f.write("\n".join(L) + "\n")


_MODEL = {"Ising": "ising", "XY": "xy", "Heisenberg": "heisenberg"}


def _lattice_inputs(p: dict):
    """(model, lattice_args positional inputs, keyword inputs) of a parameter
    file, after the checks the reference's caller makes (win.py:68-72,
    :105-113; the dipole path is refused, Lattice.py:298)."""
    model = _MODEL.get(p["modelType"])
    if model is None:
        raise ValueError("for now only Ising, XY and Heisenberg models are supported")
    if p["algorithm"] not in ("Metropolis", "Wolff"):
        raise ValueError("only the Metropolis and Wolff algorithms are supported")
    if abs(p.get("dipoleAlpha", 0.0)) > 1e-5:
        raise ValueError("dipole couplings are not supported (the reference's dipole path fails, Lattice.py:298)")
    Lx, Ly, Lz = p["LPack"]
    bonds = [(src, tgt, tuple(ov), list(J)) for (src, tgt, ov, J) in p["bondList"]]
    kw = dict(S=list(p["S"]), D=list(p["DList"]), nthermal=p["nthermal"], nsweep=p["nsweep"], tau=p["ninterval"],
              algo=1 if p["algorithm"] == "Wolff" else 0, ki=p["GcOrb"], groups=p.get("orbGroupList", []),
              group_in_sc=p.get("groupInSC", True), circuits=p.get("localCircuitList", []),
              frames=p.get("spinFrame", 0))
    return model, ((Lx, Ly, Lz), len(p["pos"]), bonds), kw


def point_args(p: dict, T: float, H: float):
    """(model, MCMainFunction tuple) of one grid point, as win.startMC /
    startMCForOn with mcMain.MC would build it (mcMain.py:16-105, :137-235).
    Built through the lattice template (numpy structure, values rescaled to
    (T, H)), which equals lattice.lattice_args bit for bit."""
    model, tmpl = grid_template(p)
    return model, tmpl.at(T, H)


def grid_template(p: dict):
    """(model, LatticeTemplate) of a parameter file: the lattice is built once
    and ``template.at(T, H)`` gives the MCMainFunction tuple of every grid
    point (equal to lattice.lattice_args at that point)."""
    from .lattice import LatticeTemplate
    model, (L, norb, bonds), kw = _lattice_inputs(p)
    return model, LatticeTemplate(model, L, norb, bonds, **kw)


def _positions(p):
    Lx, Ly, Lz = p["LPack"]
    Lm = np.asarray(p["LMatrix"], dtype=float)
    b = np.asarray(p["pos"], dtype=float)
    out = []
    for x in range(Lx):
        for y in range(Ly):
            for z in range(Lz):
                for o in range(len(b)):
                    out.append(np.dot(np.array([x, y, z]) + b[o], Lm))
    return np.array(out)


def start_simulation(rpath: str, workdir: str = ".", seed: int = 1, device: int = 0, schedule: str = "auto",
                     threads: int = 16):
    """Run the whole (T, H) grid of parameter file ``rpath`` as one batch and
    write ``out``, ``spinDotSpin.txt``, spin-frame files and ``result.txt`` in
    ``workdir`` with the reference's formats.  Point ID = iH*nT + iT gets Philox
    key seed + ID.  Returns the result.txt rows
    (T, H, <Si>, <Sj>, susceptibility, E, capacity, Q, U4, autocorrelation)."""
    from . import Batch
    p = load_param(rpath)
    TList = np.linspace(p["T0"], p["T1"], p["nT"])
    HList = np.linspace(p["H0"], p["H1"], p["nH"])
    pts = [(iH * len(TList) + iT, float(T), float(H)) for iH, H in enumerate(HList) for iT, T in enumerate(TList)]
    with open(os.path.join(workdir, "out"), "w") as f:
        f.write("#T #H\n")
    with open(os.path.join(workdir, "spinDotSpin.txt"), "w") as f:
        f.write("#T #H\n")
    # one lattice build for the whole grid; each point rescales J, D and h
    model, tmpl = grid_template(p)
    built = [(model, tmpl.at(T, H, arrays=True)) for (_, T, H) in pts]
    b = Batch(device=device)
    with ThreadPoolExecutor(max_workers=max(1, threads)) as pool:
        # adds from several threads: the engine's replica index is returned by add
        idx = list(pool.map(lambda k: b.add(built[k][0], built[k][1], seed=seed + pts[k][0], schedule=schedule),
                            range(len(pts))))
    b.run()
    res = [b.result(i) for i in idx]
    b.close()
    Lx, Ly, Lz = p["LPack"]
    N = Lx * Ly * Lz * len(p["pos"])
    xyz = _positions(p) if p.get("spinFrame", 0) > 0 else None
    rows = []
    for (ID, T0, H), (model, _), (r, ex) in zip(pts, built, res):
        T = max(T0, 0.1)  # mcMain.MC clamps; the result rows keep the grid T
        if model == "ising":
            si, sj, sij, ac, E, E2, Er, E2r, U4, stot = r[:10]
            E *= T; E2 *= T * T; Er *= T; E2r *= T * T
            with open(os.path.join(workdir, "out"), "a") as f:
                f.write("%.3f %.3f %.3f %.3f %.3f %.3f %.3f %.3f %.3f %.3f %.6f\n" %
                        (T, H, si, sj, stot, sij, E, E2, Er, E2r, U4))
            if xyz is not None:
                for k in range(p["spinFrame"]):
                    with open(os.path.join(workdir, "IsingSpinDistribution.T%.3f.H%.3f.%d.txt" % (T, H, k)), "w") as f:
                        f.write("#x       #y       #z       #spin\n")
                        fr = ex["frames"][k]
                        for i in range(N):
                            f.write("%.6f %.6f %.6f %.3f\n" % (xyz[i][0], xyz[i][1], xyz[i][2], fr[i][0]))
            rows.append((T0, H, si, sj, (sij - si * sj) / T0, E, (E2 - E * E) / T0 ** 2 * N, 0.0, U4, ac))
            continue
        (six, siy, siz, sjx, sjy, sjz, sij, ac, E, E2, U4, sirx, siry, sirz, sjrx, sjry, sjrz, sijr, Er, E2r,
         sitz, sjtz, stz, sih, sjh, sth, Q) = r[:27]
        E *= T; E2 *= T * T; Er *= T; E2r *= T * T
        spi, spj = np.array([six, siy, siz]), np.array([sjx, sjy, sjz])
        spir, spjr = np.array([sirx, siry, sirz]), np.array([sjrx, sjry, sjrz])
        li, lj = float(np.sqrt(spi @ spi)), float(np.sqrt(spj @ spj))
        with open(os.path.join(workdir, "out"), "a") as f:
            f.write("T= %.6E h= %.6E <Siz>= %.6E <Sjz>= %.6E <Sz>= %.6E <Sih>= %.6E <Sjh>= %.6E <Sh>= %.6E <Si>= %.6E "
                    "<Sj>= %.6E <SiSj>= %.6E <Si><Sj>= %.6E <E>= %.6E <E^2>= %.6E <U4>= %.6E <SiSj>r= %.6E "
                    "<Si>r<Sj>r= %.6E <Er>= %.6E <E^2_r>= %.6E <Q>= %.6E\n" %
                    (T, H, sitz, sjtz, stz, sih, sjh, sth, li, lj, sij, float(spi @ spj), E, E2, U4, sijr,
                     float(spir @ spjr), Er, E2r, Q))
        if xyz is not None:
            for k in range(p["spinFrame"]):
                with open(os.path.join(workdir, "OnSpinDistribution.T%.3f.H%.3f.%d.txt" % (T, H, k)), "w") as f:
                    f.write("#x       #y       #z       #spinx  #spiny  #spinz\n")
                    fr = ex["frames"][k]
                    for i in range(N):
                        f.write("%.6f %.6f %.6f %.6f %.6f %.6f\n" % (xyz[i][0], xyz[i][1], xyz[i][2],
                                                                     fr[i][0], fr[i][1], fr[i][2]))
        groups = r[28]
        if p.get("orbGroupList"):
            G = len(p["orbGroupList"])
            with open(os.path.join(workdir, "spinDotSpin.txt"), "a") as f:
                f.write("%.3f %.3f " % (T, H))
                for c in range((G + 1) * (G + 1) + (G + 1)):
                    f.write("%.6f " % groups[c])
                f.write("\n")
        rows.append((T0, H, li, lj, (sij - float(spi @ spj)) / T0, E, (E2 - E * E) / T0 ** 2 * N, Q, U4, ac))
    with open(os.path.join(workdir, "result.txt"), "w") as f:
        f.write("#Temp          #Field         #<Si>          #<Sj>          #Susc          #Energy(K)     "
                "#Capacity(K/K) #Topo.Q        #U4            #Auto-corr.    \n")
        for row in rows:
            f.write("%15.6E%15.6E%15.6E%15.6E%15.6E%15.6E%15.6E%15.6E%15.6E%15.6E\n" % row)
    return rows
