"""Generates the golden fixtures of tests/golden/ from the reference's own LBM
sources (compiled against the AMReX stand-in by oracle/build_ref.sh into
oracle/_ref/).  Run where the reference sources are present:

    python tests/golden/make_golden.py

Writes
  units.json   -- per tests/inputs/*.inputs: the lattice quantities the
                  reference's UnitConverter and resolveBC derive (floats as
                  float.hex strings, so comparisons are exact).
  cases.npz    -- small domains advanced by the reference code: initial
                  state, populations after init, after K steps (valid and
                  ghost-grown) and the updateMacroscopic moments.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

FACES6 = ["lox", "hix", "loy", "hiy", "loz", "hiz"]


def parse_inputs(path):
    """Minimal ParmParse reader for the fixture generator (last definition wins)."""
    toks = []
    for line in open(path):
        line = line.split("#", 1)[0]
        toks += line.replace("=", " = ").split()
    defs = {}
    i = 0
    while i < len(toks):
        key = toks[i]
        assert toks[i + 1] == "=", f"bad inputs near {key}"
        i += 2
        vals = []
        while i < len(toks) and not (i + 1 < len(toks) and toks[i + 1] == "="):
            vals.append(toks[i])
            i += 1
        defs[key] = vals
    return defs


def units_fixture(path):
    d = parse_inputs(path)
    lattice = d.get("lbm.lattice_type", ["D3Q19"])[0]
    dim, q = O.LATTICE_DQ[lattice]
    f = lambda k, dflt=None: float(d[k][0]) if k in d else dflt  # noqa: E731
    ncells = [int(x) for x in d["grid.ncells"][:dim]]
    lo = [float(x) for x in d["geometry.prob_lo"][:dim]]
    hi = [float(x) for x in d["geometry.prob_hi"][:dim]]
    accel = [float(x) for x in d.get("forcing.accel", [])] or [0.0] * dim
    rho_ref = f("units.ref_density", 1.0)
    names = [None] * 6
    for a in range(dim):
        names[2 * a] = d["bc.lo_type"][a]
        names[2 * a + 1] = d["bc.hi_type"][a]
    uw, ui, fr = [], [], []
    for fc in range(2 * dim):
        uw += [float(x) for x in d.get(f"bc.{FACES6[fc]}_Uwall", [0.0] * dim)]
        ui += [float(x) for x in d.get(f"bc.{FACES6[fc]}_Uin", [0.0] * dim)]
        fr.append(f(f"bc.{FACES6[fc]}_rho", rho_ref))
    rc, u = O.units(dim, ncells, lo, hi, ref_length=f("units.ref_length", 1.0),
                    ref_velocity=f("units.ref_velocity", 1.0), ref_density=rho_ref,
                    Re=f("units.Re"), nu_phys=f("units.nu_phys"), u_lat=f("lbm.u_lat"), tau=f("lbm.tau"),
                    accel=accel, vel=uw + ui, rho=[rho_ref] + fr, kind="ref")
    assert rc == 0, f"reference rejected {path}"
    vel = u["vel_lat"]
    uwl = vel[: len(uw)].reshape(2 * dim, dim)
    uil = vel[len(uw):].reshape(2 * dim, dim)
    rho_wall = u["rho_lat"][0]
    face_type, face_rho, face_U = [], [], []
    for fc in range(6):
        t = O.BC[names[fc]] if names[fc] else O.BC["Periodic"]
        face_type.append(t)
        r, U = 0.0, [0.0, 0.0, 0.0]
        if t != O.BC["Periodic"]:
            r = rho_wall
            if t == O.BC["MovingWall"]:
                U[:dim] = list(uwl[fc])
            elif t == O.BC["Inflow"]:
                U[:dim] = list(uil[fc])
            elif t == O.BC["PressureOutlet"]:
                r = u["rho_lat"][1 + fc]
        face_rho.append(r)
        face_U.append(U)
    force = list(u["accel_lat"]) + [0.0] * (3 - dim)
    cfg = O.Config(lattice, ncells, omega=u["omega"], faces=face_type, face_rho=face_rho, face_U=face_U,
                   force=force if any(a != 0.0 for a in accel) else None)
    rc2, types, rr, UU = O.resolve_bc(cfg, kind="ref")
    assert rc2 == 0
    hx = lambda v: float(v).hex()  # noqa: E731
    return {
        "lattice": lattice, "n": ncells, "forced": int(cfg.force is not None),
        "omega": hx(u["omega"]), "tau": hx(u["tau"]), "dx": hx(u["dx"]), "dt": hx(u["dt"]),
        "u_lat": hx(u["u_lat"]), "nu_lat": hx(u["nu_lat"]),
        "force": [hx(x) for x in force], "face_type": face_type, "face_rho": [hx(x) for x in face_rho],
        "face_U": [[hx(x) for x in U] for U in face_U],
        "bc_type": [int(t) for t in types], "bc_rho": [hx(x) for x in rr],
        "bc_U": [[hx(x) for x in row] for row in UU],
    }


def cases():
    """(name, Config, init kind, steps)."""
    rng = np.random.default_rng(20261203)
    P, NS, MW, IN, OF, PO = "Periodic", "NoSlip", "MovingWall", "Inflow", "Outflow", "PressureOutlet"
    out = []
    for lat, n in (("D2Q9", (12, 10)), ("D3Q15", (5, 4, 4)), ("D3Q19", (5, 4, 4)), ("D3Q27", (5, 4, 4))):
        dim = O.LATTICE_DQ[lat][0]
        z = [P, P] if dim == 3 else [P, P]
        sets = {
            "periodic": [P, P, P, P] + z,
            "channel": [P, P, NS, NS] + z,
            "cavity": ([NS, NS, NS, MW] + [P, P]) if dim == 2 else [NS, NS, NS, NS, NS, MW],
            "inflow_po": [IN, PO, NS, NS] + z,
            "inflow_of": [IN, OF, P, P] + ([NS, MW] if dim == 3 else [P, P]),
            "mixed": ([OF, PO, MW, NS] + [P, P]) if dim == 2 else [OF, PO, P, P, MW, NS],
        }
        for sname, faces in sets.items():
            for forced in (False, True):
                U = [[0.0, 0.0, 0.0] for _ in range(6)]
                for fc in range(2 * dim):
                    if faces[fc] == MW:
                        for c in range(dim):
                            if c != fc // 2:
                                U[fc][c] = float(rng.uniform(-0.08, 0.08))
                    if faces[fc] == IN:
                        U[fc][fc // 2] = float(rng.uniform(0.01, 0.05)) * (1 if fc % 2 == 0 else -1)
                rho_f = [1.0 if faces[fc] != PO else float(rng.uniform(0.98, 1.02)) for fc in range(6)]
                force = tuple(float(x) for x in rng.uniform(-2e-4, 2e-4, 3)) if forced else None
                if force and dim == 2:
                    force = (force[0], force[1], 0.0)
                omega = float(1.0 / rng.uniform(0.52, 1.6))
                cfg = O.Config(lat, n, omega=omega, faces=faces, face_rho=rho_f, face_U=U, force=force)
                kind = "fields" if sname != "mixed" else "random_f"
                out.append((f"{lat}_{sname}_{'F' if forced else 'U'}", cfg, kind, 9))
    return out


def main():
    if not O.ref_available() and not O.build_ref():
        raise SystemExit("reference sources unavailable: cannot generate golden fixtures")
    units = {}
    for fn in sorted(os.listdir(os.path.join(ROOT, "tests", "inputs"))):
        if fn.endswith(".inputs"):
            units[fn] = units_fixture(os.path.join(ROOT, "tests", "inputs", fn))
    with open(os.path.join(HERE, "units.json"), "w") as fh:
        json.dump(units, fh, indent=1, sort_keys=True)
    rng = np.random.default_rng(7)
    arrays = {}
    index = []
    for name, cfg, kind, steps in cases():
        sim = O.OracleSim(cfg, "ref")
        N = sim.N
        if kind == "fields":
            rho0 = 1.0 + 0.02 * rng.standard_normal(N)
            u0 = 0.04 * rng.standard_normal(cfg.dim * N)
            rho_i, u_i = sim.init_fields(rho0, u0)
            arrays[name + "/rho0"], arrays[name + "/u0"] = rho0, u0
            arrays[name + "/rho_init"], arrays[name + "/u_init"] = rho_i, u_i
        else:
            f0 = rng.uniform(0.5, 1.5, cfg.q * N) / cfg.q
            sim.set_f(f0)
            sim.fill_ghosts()
            arrays[name + "/f0"] = f0
        arrays[name + "/f_init"] = sim.get_f()
        sim.step(steps)
        arrays[name + "/f_final"] = sim.get_f()
        arrays[name + "/fg_final"] = sim.get_f_ghost()
        r, u = sim.moments()
        arrays[name + "/rho_final"], arrays[name + "/u_final"] = r, u
        index.append({"name": name, "lattice": cfg.lattice, "n": list(cfg.n), "omega": cfg.omega.hex(),
                      "faces": [O.BC[f] for f in cfg.faces], "face_rho": [x.hex() for x in cfg.face_rho],
                      "face_U": [[x.hex() for x in U] for U in cfg.face_U],
                      "force": [x.hex() for x in cfg.force] if cfg.force else None,
                      "kind": kind, "steps": steps})
    arrays["index"] = np.array(json.dumps(index))
    np.savez_compressed(os.path.join(HERE, "cases.npz"), **arrays)
    print(f"wrote {len(index)} cases, {len(units)} unit fixtures")


if __name__ == "__main__":
    main()
