"""DL_POLY 2 input decks (CONTROL, FIELD, CONFIG) of this fork, read into the inputs of
mbx_water_step, so that a deck prepared for the reference drives the GB300 path unchanged.

Only what the MB-pol force path reads is taken; other keywords are skipped, as the
reference skips what its run does not use.
- CONTROL (SOURCE/simdef_cmd.f):
  - `cut`, `rvdw`, `delr`;
  - `ewald sum alpha k1 k2 k3`, or `ewald precision eps` with alpha and kmax from the cell
    (:1213-1300);
  - `spme` is read like `ewald` (this library evaluates it with the Ewald sum);
  - `polar`, `iter toler` (Debye), `aspc_omega`, `ascc`, `ascd`;
  - `aspc` (ASPC on, k 4, 6 converged steps, SOR weight 6/11) and `aspc_k k` (for k 2 or
    4: weight (k+2)/(2k+3), k+2 converged steps; ASPC stays off without `aspc`), read in the
    order the lines come (:742-788);
  - `vmbpol` (:1040-1060: Thole 0.055 / 0.626 / 0.055, smearing 0.4 / 0.4, gamma
    0.426706882);
  - `eps` (dielectric constant).
- FIELD (SOURCE/sysdef_cmd.f):
  - `units ev|kcal|kj|internal` (:204-232);
  - molecule types with `nummols` and `atoms` lines: name, mass, charge, then with
    `polar` in CONTROL polar and polar2, then repeat (:355-420);
  - `vdw` pairs with the key `tt68`, type 12: C6 a6 C8 a8, with C6 and C8 times the energy
    unit (:1442-1590).

  The last molecule type holds the M sites (SOURCE/dlpoly_cmd.f:931-941).
- CONFIG: title, `levcfg imcon`, three cell vectors when imcon > 0, then per atom a name
  line, positions, velocities (levcfg >= 1) and forces (levcfg >= 2).

Readers take a path or the file's text.
"""
import io
import math
import os
import re

import numpy as np

EATD = 4.803239                     # Debye per e Angstrom (SOURCE/module.f90:38)
ENGUNIT = {"ev": 9648.530821, "kcal": 418.4, "kj": 1.0e2, "internal": 1.0}
_NUM = re.compile(r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eEdD][-+]?\d+)?")


def _lines(src):
    if isinstance(src, io.IOBase):
        return src.read().splitlines()
    if isinstance(src, str) and "\n" not in src and os.path.exists(src):
        with open(src) as f:
            return f.read().splitlines()
    return str(src).splitlines()


def _numbers(text):
    """the numbers of a record in order (Fortran d exponents accepted), as dblstr finds them"""
    return [float(t.replace("d", "e").replace("D", "e")) for t in _NUM.findall(text)]


def _fields(line):
    return line.split()


def read_control(src):
    """CONTROL keywords of the MB-pol path -> dict"""
    c = {"rcut": None, "rvdw": None, "delr": 0.0, "ewald": None, "polar": False, "toler": None,
         "sor_omega": 0.3, "ascc": None, "ascd": None, "vmbpol": False, "epsq": 1.0, "spme": False,
         "aspc": False, "aspc_k": 4, "aspc_iter_nstep": 6}
    for raw in _lines(src):
        rec = raw.strip().lower()
        if not rec or rec.startswith("#"):
            continue
        nums = _numbers(rec)
        if rec.startswith("finish"):
            break
        if rec.startswith("cut"):
            c["rcut"] = nums[0]
        elif rec.startswith("rvdw"):
            c["rvdw"] = nums[0]
        elif rec.startswith("delr"):
            c["delr"] = nums[0]
        elif rec.startswith("ewald") or rec.startswith("spme"):
            c["spme"] = rec.startswith("spme")
            if "precision" in rec:
                c["ewald"] = ("precision", nums[0])
            else:
                c["ewald"] = ("sum", nums[0], int(nums[1]), int(nums[2]), int(nums[3]))
        elif rec.startswith("polar"):
            c["polar"] = True
        elif rec.startswith("iter"):
            c["toler"] = nums[0] / EATD        # Debye to e Angstrom
        elif rec.startswith("aspc_omega"):
            if not 0.0 <= nums[0] <= 1.0:
                raise ValueError("CONTROL: aspc_omega must lie in [0, 1]")
            c["sor_omega"] = nums[0]
        elif rec.startswith("aspc_k"):
            # Kolafa's corrector weight and iter_nstep = k+2 for k = 2 or 4 (SOURCE/simdef_cmd.f:754-773)
            k = int(nums[0])
            if k < 0:
                raise ValueError("CONTROL: aspc_k must be >= 0")
            c["aspc_k"] = k
            if k in (2, 4):
                c["sor_omega"] = (k + 2.0) / (2.0 * k + 3.0)
                c["aspc_iter_nstep"] = k + 2
        elif rec.startswith("aspc"):
            # ASPC on with k = 4 (SOURCE/simdef_cmd.f:775-788)
            c["aspc"] = True
            c["sor_omega"] = 6.0 / 11.0
            c["aspc_k"] = 4
            c["aspc_iter_nstep"] = 6
        elif rec.startswith("ascc"):
            c["ascc"] = nums[0]
        elif rec.startswith("ascd"):
            c["ascd"] = nums[0]
        elif rec.startswith("vmbpol"):
            c["vmbpol"] = True
        elif re.match(r"eps\b", rec) or rec.startswith("eps "):
            c["epsq"] = nums[0]
    return c


def read_field(src, polar=True):
    """FIELD -> dict(engunit, molecules=[(name, nummols, [(site, mass, charge, polar, polar2)])],
    vdw=[(atom1, atom2, key, params in internal units)])"""
    lines = [l for l in _lines(src)]
    out = {"engunit": 1.0, "molecules": [], "vdw": []}
    i = 1   # the first line is the title
    while i < len(lines):
        f = _fields(lines[i])
        key = f[0].lower() if f else ""
        if key == "units":
            u = f[1].lower() if len(f) > 1 else "internal"
            if u not in ENGUNIT:
                raise ValueError("FIELD: unknown energy unit %r" % u)
            out["engunit"] = ENGUNIT[u]
        elif key.startswith("molecules") or key.startswith("molecular"):
            nmol = int(_numbers(lines[i])[0])
            i += 1
            for _ in range(nmol):
                name = _fields(lines[i])[0]
                i += 1
                nummols, sites = 0, []
                while i < len(lines):
                    g = _fields(lines[i])
                    k = g[0].lower() if g else ""
                    if k == "nummols":
                        nummols = int(g[1])
                    elif k == "atoms":
                        nsite = int(g[1])
                        got = 0
                        while got < nsite:
                            i += 1
                            a = _fields(lines[i])
                            mass, charge = float(a[1]), float(a[2])
                            if polar:
                                pol = float(a[3]) if len(a) > 3 else 0.0
                                pol2 = float(a[4]) if len(a) > 4 else 0.0
                                rep = int(a[5]) if len(a) > 5 else 1
                            else:
                                pol = pol2 = 0.0
                                rep = int(a[3]) if len(a) > 3 else 1
                            rep = rep or 1
                            sites += [(a[0], mass, charge, pol, pol2)] * rep
                            got += rep
                    elif k == "finish":
                        break
                    i += 1
                out["molecules"].append((name, nummols, sites))
                i += 1
            continue
        elif key == "vdw":
            n = int(f[1])
            for _ in range(n):
                i += 1
                g = _fields(lines[i])
                k = g[2].lower()
                p = [float(x.replace("d", "e").replace("D", "e")) for x in g[3:]]
                if k == "tt68":   # C6 a6 C8 a8: C6 and C8 in the energy unit
                    p = p + [0.0] * (4 - len(p))
                    p[0] *= out["engunit"]
                    p[2] *= out["engunit"]
                out["vdw"].append((g[0], g[1], k, p))
        elif key == "close":
            break
        i += 1
    return out


def read_config(src):
    """CONFIG -> dict(title, levcfg, imcon, cell[9], names, xyz[n,3], vel[n,3] or None)"""
    lines = _lines(src)
    head = _fields(lines[1])
    levcfg, imcon = int(head[0]), int(head[1])
    i = 2
    cell = np.zeros(9)
    if imcon > 0:
        for k in range(3):
            cell[3 * k:3 * k + 3] = _numbers(lines[i])[:3]
            i += 1
    names, xyz, vel = [], [], []
    while i < len(lines) and lines[i].strip():
        names.append(_fields(lines[i])[0])
        xyz.append(_numbers(lines[i + 1])[:3])
        i += 2
        if levcfg >= 1:
            vel.append(_numbers(lines[i])[:3])
            i += 1
        if levcfg >= 2:
            i += 1
    return {"title": lines[0], "levcfg": levcfg, "imcon": imcon, "cell": cell, "names": names,
            "xyz": np.array(xyz, np.float64).reshape(-1, 3),
            "vel": np.array(vel, np.float64).reshape(-1, 3) if levcfg >= 1 else None}


def ewald_from_precision(cell, rcut, eps, imcon=1):
    """alpha and kmax of `ewald precision eps` (SOURCE/simdef_cmd.f:1270-1290): from the
    cutoff and the lengths of the cell vectors"""
    a = np.asarray(cell, np.float64)
    lengths = [math.sqrt(a[0] ** 2 + a[1] ** 2 + a[2] ** 2), math.sqrt(a[3] ** 2 + a[4] ** 2 + a[5] ** 2),
               math.sqrt(a[6] ** 2 + a[7] ** 2 + a[8] ** 2)]
    eps = min(abs(eps), 0.5)
    tol = math.sqrt(abs(math.log(eps * rcut)))
    alpha = math.sqrt(abs(math.log(eps * rcut * tol))) / rcut
    tol1 = math.sqrt(-math.log(eps * rcut * (2.0 * tol * alpha) ** 2))
    fac = 2.0 ** (1.0 / 3.0) if imcon in (4, 5, 7) else 1.0
    # Fortran nint: half away from zero
    km = [int(math.floor(abs(x) + 0.5)) * (1 if x >= 0 else -1)
          for x in (0.25 + fac * L * alpha * tol1 / math.pi for L in lengths)]
    return alpha, km


def deck_inputs(control, field, config):
    """The inputs of mbx_water_step (and mbx_disp_setup) from read_control / read_field /
    read_config results.  Standard layout: the water molecule type(s) of 3 sites first, the
    M-site type last (one site per water).  Returns dict(nw, natms, imcon, cell, xyz, vel,
    mass, polr, polr2, polar_prm[15], disp=(ntypes, prm) or None, ltype, molecule (0-based
    ids, one per water), rvdw, delr, aspc=(k, iter_nstep) or None: mbx_set_aspc's
    arguments)."""
    mols = field["molecules"]
    if len(mols) < 2 or len(mols[-1][2]) != 1:
        raise ValueError("FIELD: expected the water type(s) then a one-site M-site type")
    water = [m for m in mols[:-1]]
    nw = sum(m[1] for m in water if len(m[2]) == 3)
    if any(len(m[2]) != 3 for m in water) or mols[-1][1] != nw:
        raise ValueError("FIELD: only 3-site waters and one M site per water are on this path")
    sites, molecule = [], []
    mol = 0
    for name, nummols, s in water:
        for _ in range(nummols):
            mol += 1
            sites += s
            molecule += [mol] * 3
    sites += mols[-1][2] * nw
    molecule += list(range(1, nw + 1))
    n = len(sites)
    if config["xyz"].shape[0] != n:
        raise ValueError("CONFIG has %d atoms, FIELD %d sites" % (config["xyz"].shape[0], n))
    polr = np.array([s[3] for s in sites], np.float64)
    polr2 = np.array([s[4] for s in sites], np.float64)
    mass = np.array([s[1] for s in sites], np.float64)
    cell = config["cell"]
    rcut = control["rcut"]
    if rcut is None:
        raise ValueError("CONTROL: no cut")
    ew = control["ewald"]
    if ew is None:
        raise ValueError("CONTROL: no ewald or spme line")
    if ew[0] == "precision":
        alpha, km = ewald_from_precision(cell, rcut, ew[1], config["imcon"])
    else:
        alpha, km = ew[1], list(ew[2:5])
    mb = control["vmbpol"]
    ascc = control["ascc"] if control["ascc"] is not None else (0.4 if mb else 0.0)
    ascd = control["ascd"] if control["ascd"] is not None else (0.4 if mb else 0.0)
    toler = control["toler"] if control["toler"] is not None else 1e-8 / EATD
    prm = np.array([alpha, rcut, control["epsq"], toler, control["sor_omega"], 0.055, 0.626, 0.055, ascc, ascd,
                    0.426706882, km[0], km[1], km[2], 22581], np.float64)
    # dispersion: tt68 pairs over the unique site names (types in first-seen order)
    names = []
    for s in sites:
        if s[0] not in names:
            names.append(s[0])
    ltype = np.zeros(n, np.int32)
    disp = None
    vdw = [v for v in field["vdw"] if v[2] == "tt68"]
    if vdw:
        nt = len(names)
        pp = np.zeros((nt * (nt + 1) // 2, 4))
        for a1, a2, _, p in vdw:
            i, j = names.index(a1) + 1, names.index(a2) + 1
            i, j = max(i, j), min(i, j)
            pp[i * (i - 1) // 2 + j - 1] = p[:4]
        used = set()
        for a1, a2, _, p in vdw:
            if any(p[:4]):
                used.update((a1, a2))
        ltype = np.array([names.index(s[0]) + 1 if s[0] in used else 0 for s in sites], np.int32)
        disp = (nt, pp)
    return {"nw": nw, "natms": n, "imcon": config["imcon"], "cell": cell, "xyz": config["xyz"],
            "vel": config["vel"], "mass": mass, "polr": polr, "polr2": polr2, "polar_prm": prm, "disp": disp,
            "ltype": ltype, "molecule": np.array(molecule, np.int32) - 1, "rvdw": control["rvdw"] or rcut,
            "delr": control["delr"],
            "aspc": (control["aspc_k"], control["aspc_iter_nstep"]) if control.get("aspc") else None}


def write_deck(box, control_extra="", units="kcal", vdw=None, title="MB-pol water"):
    """(CONTROL, FIELD, CONFIG) text for a WaterBox in the standard layout, with MB-pol's
    polarizabilities: O and M 1.310, H 0.294 (polar2 0 on the M site); vdw is a list of
    (name1, name2, C6, a6, C8, a8) in `units`."""
    nw = box.nw
    control = "\n".join([title, "polar", "vmbpol", "cut 9.0", "delr 1.0", "ewald sum 0.3 8 8 8",
                         "iter 1.0e-8", control_extra, "finish"]) + "\n"
    vdw = vdw or []
    field = [title, "units %s" % units, "molecules 2", "water", "nummols %d" % nw, "atoms 3",
             "OW 15.9994 0.0 1.310 1.310 1", "HW 1.00794 0.0 0.294 0.294 2", "finish", "msite",
             "nummols %d" % nw, "atoms 1", "MW 0.0 0.0 1.310 0.0 1", "finish", "vdw %d" % len(vdw)]
    field += ["%s %s tt68 %.17g %.17g %.17g %.17g" % v for v in vdw]
    field += ["close"]
    imcon = box.imcon
    cfg = [title, "%10d%10d" % (1, imcon)]
    c = np.asarray(box.cell, np.float64)
    for k in range(3):
        cfg.append("%.17g %.17g %.17g" % tuple(c[3 * k:3 * k + 3]))
    names = ["OW", "HW", "HW"] * nw + ["MW"] * nw
    for i, nm in enumerate(names):
        cfg.append("%-8s%10d" % (nm, i + 1))
        cfg.append("%.17g %.17g %.17g" % tuple(box.xyz[i]))
        cfg.append("%.17g %.17g %.17g" % tuple(box.vel[i]))
    return control, "\n".join(field) + "\n", "\n".join(cfg) + "\n"


def read_deck(control, field, config):
    """read_control + read_field (its atom columns by CONTROL's `polar`) + read_config, then
    deck_inputs"""
    c = read_control(control)
    return deck_inputs(c, read_field(field, polar=c["polar"]), read_config(config))
