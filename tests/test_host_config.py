"""Host side of the boundary: the inputs reader, unit chain and BC resolution
of libmph against values the reference's own code derived (tests/golden/
units.json) and against the oracle; the reference's abort cases become error
codes.  No GPU needed."""
import os
import re

import numpy as np
import pytest

import golden_cases as G

INPUTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "inputs")


@pytest.mark.parametrize("fn", sorted(G.units().keys()))
def test_derive_matches_reference_units_bitwise(fn, mph):
    exp = G.units()[fn]
    ip = mph.InputParser(os.path.join(INPUTS, fn))
    d, info = ip.derive()
    hx = lambda v: float(v).hex()  # noqa: E731
    assert (d.dim, d.q) == mph.LATTICE_DQ[exp["lattice"]]
    assert list(d.n)[: d.dim] == exp["n"]
    assert hx(d.omega) == exp["omega"]
    assert hx(info.tau) == exp["tau"] and hx(info.dx) == exp["dx"] and hx(info.dt) == exp["dt"]
    assert hx(info.u_lat) == exp["u_lat"] and hx(info.nu_lat) == exp["nu_lat"]
    assert d.forced == exp["forced"]
    if d.forced:
        assert [hx(x) for x in d.force] == exp["force"]
    assert list(d.face_type) == exp["face_type"]
    for f in range(6):
        if exp["face_type"][f] != 5:
            assert hx(d.face_rho[f]) == exp["face_rho"][f]
            assert [hx(x) for x in d.face_U[f]] == exp["face_U"][f]
    tab = mph.resolve_bc(d)
    ntab = 27 if d.dim == 3 else 9
    for c in range(ntab):
        t, r, U = tab[c]
        assert t == exp["bc_type"][c]
        if t != 5:
            assert hx(r) == exp["bc_rho"][c]
            assert [hx(x) for x in U] == exp["bc_U"][c]


def test_reference_inputs_files_parse(mph, oracle_mod):
    """The reference's own inputs files (read where they lie) derive the same
    omega and force as the oracle's unit chain."""
    ref = oracle_mod.REFERENCE_ROOT
    files = []
    for dp, _, fns in os.walk(ref):
        files += [os.path.join(dp, f) for f in fns if re.match(r"inputs(\.\w+|3d.*|_\w+)?$", f)]
    if not files:
        pytest.skip("reference inputs files not present on this host")
    for path in files:
        ip = mph.InputParser(path)
        d, info = ip.derive()
        lat = ip.get("lbm.lattice_type") or "D3Q19"
        dim = mph.LATTICE_DQ[lat][0]
        g = lambda k: ip.get(k)  # noqa: E731
        fl = lambda k: float(g(k).split()[0]) if g(k) else None  # noqa: E731
        rc, u = oracle_mod.units(dim, [int(x) for x in g("grid.ncells").split()[:dim]],
                                 [float(x) for x in g("geometry.prob_lo").split()[:dim]],
                                 [float(x) for x in g("geometry.prob_hi").split()[:dim]],
                                 ref_length=fl("units.ref_length") or 1.0,
                                 ref_velocity=fl("units.ref_velocity") or 1.0,
                                 ref_density=fl("units.ref_density") or 1.0, Re=fl("units.Re"),
                                 nu_phys=fl("units.nu_phys"), u_lat=fl("lbm.u_lat"), tau=fl("lbm.tau"),
                                 accel=[float(x) for x in (g("forcing.accel") or "").split()])
        assert rc == 0, path
        assert d.omega == u["omega"], path
        if d.forced:
            assert list(d.force)[:dim] == list(u["accel_lat"]), path


def test_overrides_last_definition_wins(mph):
    path = os.path.join(INPUTS, "tgv2d.inputs")
    ip = mph.InputParser(path, overrides=["lbm.tau=0.9", "grid.ncells = 32 16", "geometry.prob_hi=32 16"])
    d, info = ip.derive()
    assert abs(info.tau - 0.9) < 1e-15 and list(d.n)[:2] == [32, 16]
    assert ip.get("lbm.tau") == "0.9"


def _err(mph, text, overrides=()):
    ip = mph.InputParser(text=text, overrides=list(overrides))
    with pytest.raises(mph.MphError) as e:
        ip.derive()
    return e.value.code


BASE = """grid.ncells = 8 8
sim.max_step = 10
lbm.lattice_type = D2Q9
units.Re = 10
geometry.prob_lo = 0 0
geometry.prob_hi = 1 1
bc.lo_type = Periodic NoSlip
bc.hi_type = Periodic NoSlip
"""


def test_reference_abort_cases_become_error_codes(mph):
    assert _err(mph, BASE + "units.nu_phys = 0.1\n") == 2           # Re and nu_phys both
    assert _err(mph, BASE.replace("units.Re = 10\n", "")) == 2        # neither
    assert _err(mph, BASE + "lbm.tau = 0.8\nlbm.u_lat = 0.05\n") == 2  # tau and u_lat
    assert _err(mph, BASE + "lbm.tau = 2.5\n") == 2                   # tau out of (0.5, 2)
    assert _err(mph, BASE + "lbm.u_lat = 0.35\n") == 2                # Mach limit
    assert _err(mph, BASE + "lbm.collision_model = TRT\n") == 4       # recognised, not implemented
    assert _err(mph, BASE + "lbm.collision_model = XYZ\n") == 2
    assert _err(mph, BASE + "lbm.lattice_type = D2Q7\n") == 2
    assert _err(mph, BASE + "geometry.prob_hi = 2 1\n") == 2          # non-square lattice
    assert _err(mph, BASE + "bc.hiy_Uwall = 0.1 0.1\n") == 2          # normal wall velocity
    assert _err(mph, BASE + "bc.lo_type = Periodic Inflow\nbc.loy_Uin = 0.1 0.1\n") == 2  # tangential inflow
    assert _err(mph, BASE + "bc.lo_type = NoSlip NoSlip\nbc.hi_type = Periodic NoSlip\n") == 2
    assert _err(mph, BASE + "bc.lo_type = Outflow NoSlip\nbc.hi_type = NoSlip PressureOutlet\n") == 2
    assert _err(mph, BASE + "bc.lo_type = Outflow PressureOutlet\nbc.hi_type = NoSlip NoSlip\n") == 2
    assert _err(mph, BASE + "forcing.accel = 1 2 3\n") == 2
    assert _err(mph, BASE + "bc.loy_rho = -1\n") == 2
    assert _err(mph, BASE + "geometry.use_eb = 1\n") == 4
    assert _err(mph, BASE.replace("sim.max_step = 10\n", "")) == 5   # required key
    assert _err(mph, BASE + "lbm.tau = abc\n") == 5


def test_parse_errors(mph):
    with pytest.raises(mph.MphError) as e:
        mph.InputParser(text="grid.ncells 8 8\n")
    assert e.value.code == 5
    with pytest.raises(mph.MphError):
        mph.InputParser(path="/nonexistent/inputs")


@pytest.mark.parametrize("seed", range(12))
def test_resolve_table_matches_oracle_random_faces(seed, mph, oracle_mod):
    rng = np.random.default_rng(seed)
    names = ["MovingWall", "NoSlip", "Inflow", "Outflow", "PressureOutlet", "Periodic"]
    for lat in ("D2Q9", "D3Q19"):
        dim = mph.LATTICE_DQ[lat][0]
        faces = []
        for a in range(3):
            if a >= dim:
                faces += ["Periodic", "Periodic"]
                continue
            lo = names[rng.integers(0, 6)]
            hi = "Periodic" if lo == "Periodic" and rng.random() < 0.8 else names[rng.integers(0, 5)]
            faces += [lo, hi]
        rho = list(rng.uniform(0.9, 1.1, 6))
        U = [list(rng.uniform(-0.1, 0.1, 3)) for _ in range(6)]
        d = mph.make_desc(lat, (4, 4, 4) if dim == 3 else (4, 4), 1.0, faces=faces, face_rho=rho, face_U=U)
        cfg = oracle_mod.Config(lat, (4, 4, 4) if dim == 3 else (4, 4), omega=1.0, faces=faces, face_rho=rho,
                                face_U=U)
        rc, t, r, UU = oracle_mod.resolve_bc(cfg)
        if rc != 0:
            with pytest.raises(mph.MphError):
                mph.resolve_bc(d)
            continue
        tab = mph.resolve_bc(d)
        for c in range(27 if dim == 3 else 9):
            assert tab[c][0] == t[c]
            if t[c] != 5:
                assert tab[c][1] == r[c] and list(tab[c][2]) == list(UU[c])
