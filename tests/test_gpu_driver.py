"""The host driver (mph_run, the counterpart of the reference's main.cpp):
plot output in physical units equal to the library's moments, checkpoint /
restart bit for bit (as the reference's test_restart), stop-time handling and
error reporting."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
INPUTS = os.path.join(HERE, "inputs", "cavity2d.inputs")


def _run(mph, cwd, *over, check=True):
    exe = os.path.join(os.path.dirname(mph.__file__), "_build", "mph_run")
    r = subprocess.run([exe, INPUTS, "grid.ncells=32 32", *over], cwd=cwd, capture_output=True, text=True)
    if check:
        assert r.returncode == 0, r.stderr
    return r


def _load_npy(path):
    return np.load(path)


def test_plotfile_matches_library_moments(mph, tmp_path):
    _run(mph, tmp_path, "sim.max_step=40", "amr.plot_int=20", "amr.chk_int=0")
    d, info = mph.InputParser(INPUTS, overrides=["grid.ncells=32 32"]).derive("f64")
    s = mph.Simulation(d, info)
    s.initialize()
    s.advance(21)  # loop steps 0..20 inclusive
    rho, u = s.update_macroscopic()
    got = _load_npy(tmp_path / "plt0000020" / "density.npy")
    assert got.shape == (32, 32)
    assert np.array_equal(got.reshape(-1), rho * info.ref_density)
    vx = _load_npy(tmp_path / "plt0000020" / "vx.npy").reshape(-1)
    assert np.array_equal(vx, u[:1024] * (info.dx / info.dt))
    hdr = (tmp_path / "plt0000020" / "Header").read_text().split("\n")
    assert hdr[0] == "muphfasa_gb300_plotfile_v1" and hdr[1] == "3" and int(hdr[7]) == 20


@pytest.mark.parametrize("precision", ["f64", "f64x"])
def test_restart_is_bit_exact(mph, tmp_path, precision):
    a, b = tmp_path / "a", tmp_path / "b"
    a.mkdir()
    b.mkdir()
    p = f"mph.precision={precision}"
    _run(mph, a, p, "sim.max_step=40", "amr.plot_int=0", "amr.chk_int=20")
    _run(mph, b, p, "sim.max_step=20", "amr.plot_int=0", "amr.chk_int=20")
    _run(mph, b, p, "sim.max_step=40", "amr.plot_int=0", "amr.chk_int=20", f"amr.restart={b / 'chk0000020'}")
    fa = np.fromfile(a / "chk0000040" / "f.f64", dtype="<f8")
    fb = np.fromfile(b / "chk0000040" / "f.f64", dtype="<f8")
    assert fa.size == 9 * 32 * 32 and np.array_equal(fa, fb)
    ha = (a / "chk0000040" / "Header").read_text().split("\n")
    hb = (b / "chk0000040" / "Header").read_text().split("\n")
    assert ha == hb and ha[0] == "muphfasa_gb300_checkpoint_v1" and float(ha[2]) == 41.0
    assert ha[6] == f"mph.precision={precision}"
    ra = (a / "chk0000040" / "state.raw").read_bytes()
    assert ra == (b / "chk0000040" / "state.raw").read_bytes()


def test_errors_are_reported(mph, tmp_path):
    r = _run(mph, tmp_path, "amr.restart=nonexistent", check=False)
    assert r.returncode == 1 and "no Header file" in r.stderr
    r = _run(mph, tmp_path, "mph.precision=f128", check=False)
    assert r.returncode == 1 and "mph.precision" in r.stderr


def _inputs_variant(path, **keys):
    """cavity2d.inputs with some keys replaced."""
    lines = []
    for line in open(INPUTS).read().splitlines():
        k = line.split("=")[0].strip()
        if k in keys:
            continue
        lines.append(line)
    lines += [f"{k} = {v}" for k, v in keys.items()]
    path.write_text("\n".join(lines) + "\n")
    return str(path)


def test_batch_runner_equals_single_runs(mph, tmp_path):
    """mph_batch_run over three cavities of different size, Re and length
    writes, per domain, the plot directories mph_run writes for that inputs
    file alone (FP64 batch = single handles, bit for bit) and a final one."""
    exe = os.path.join(os.path.dirname(mph.__file__), "_build", "mph_batch_run")
    run = os.path.join(os.path.dirname(mph.__file__), "_build", "mph_run")
    cases = [dict(**{"grid.ncells": "24 24", "sim.max_step": 30, "units.Re": 100.0, "amr.plot_int": 15}),
             dict(**{"grid.ncells": "32 40", "geometry.prob_hi": "1.0 1.25", "sim.max_step": 45, "units.Re": 120.0,
                     "amr.plot_int": 15}),
             dict(**{"grid.ncells": "40 32", "geometry.prob_hi": "1.25 1.0", "sim.max_step": 60, "units.Re": 50.0,
                     "amr.plot_int": 15})]
    files = [_inputs_variant(tmp_path / f"case{i}.inputs", **c) for i, c in enumerate(cases)]
    r = subprocess.run([exe, *files, f"mph.out={tmp_path / 'out'}", "amr.chk_int=0"], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert len([ln for ln in r.stdout.splitlines() if ln.startswith("domain ")]) == 3
    for i, (f, c) in enumerate(zip(files, cases)):
        single = tmp_path / f"single{i}"
        single.mkdir()
        r1 = subprocess.run([run, f, "amr.chk_int=0"], cwd=single, capture_output=True, text=True)
        assert r1.returncode == 0, r1.stderr
        dom = tmp_path / "out" / f"domain{i:04d}"
        for step in range(0, c["sim.max_step"] + 1, 15):
            for var in ("density", "vx", "vy"):
                a = np.load(dom / f"plt{step:07d}" / f"{var}.npy")
                b = np.load(single / f"plt{step:07d}" / f"{var}.npy")
                assert np.array_equal(a, b), (i, step, var)
            assert (dom / f"plt{step:07d}" / "Header").read_text() == (single / f"plt{step:07d}" / "Header").read_text()
        last = c["sim.max_step"]
        for var in ("density", "vx", "vy"):
            assert np.array_equal(np.load(dom / "final" / f"{var}.npy"), np.load(single / f"plt{last:07d}" / f"{var}.npy"))


def test_batch_runner_stops_converged_domains(mph, tmp_path):
    """With mph.tol each domain stops at the first residual check below it;
    its final fields are those of a single handle advanced as many steps."""
    exe = os.path.join(os.path.dirname(mph.__file__), "_build", "mph_batch_run")
    files = [_inputs_variant(tmp_path / "a.inputs", **{"grid.ncells": "16 16", "units.Re": 10.0}),
             _inputs_variant(tmp_path / "b.inputs", **{"grid.ncells": "24 24", "units.Re": 20.0})]
    r = subprocess.run([exe, *files, f"mph.out={tmp_path / 'out'}", "mph.tol=1e-4", "mph.check_every=50",
                        "sim.max_step=200000", "amr.plot_int=0", "mph.precision=f64"], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = [ln.split() for ln in r.stdout.splitlines() if ln.startswith("domain ")]
    assert len(lines) == 2
    for i, (ln, f) in enumerate(zip(lines, files)):
        steps, res = int(ln[ln.index("steps") + 1]), float(ln[ln.index("residual") + 1])
        assert "converged" in ln and steps % 50 == 0 and steps < 200000 and res < 1e-4
        d, info = mph.InputParser(f, overrides=["sim.max_step=200000"]).derive("f64")
        s = mph.Simulation(d, info)
        s.initialize()
        s.advance(steps)
        rho, _ = s.update_macroscopic()
        got = np.load(tmp_path / "out" / f"domain{i:04d}" / "final" / "density.npy").reshape(-1)
        assert np.array_equal(got, rho * info.ref_density)


def test_batch_runner_fixed_point_converges_and_drops_a_diverging_domain(mph, tmp_path):
    """mph_batch_run in the FP64-accurate fixed point: a stable cavity stops at
    its first residual check below 1e-8 with the fields of a single f64x
    handle advanced as many steps, bit for bit, while a cavity with tau =
    0.5001 at Re = 72 000 (lid at 0.1 in lattice units, a grid Reynolds number
    of 3000: unstable) leaves the fixed-point range, is reported as diverged
    and does not stop the run."""
    exe = os.path.join(os.path.dirname(mph.__file__), "_build", "mph_batch_run")
    files = [_inputs_variant(tmp_path / "a.inputs", **{"grid.ncells": "16 16", "units.Re": 10.0}),
             _inputs_variant(tmp_path / "b.inputs", **{"grid.ncells": "24 24", "lbm.tau": 0.5001,
                                                       "units.Re": 72000.0})]
    r = subprocess.run([exe, *files, f"mph.out={tmp_path / 'out'}", "mph.tol=1e-8", "mph.check_every=500",
                        "sim.max_step=400000", "amr.plot_int=0", "mph.precision=f64x"], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = {int(ln.split()[1]): ln for ln in r.stdout.splitlines() if ln.startswith("domain ")}
    assert "diverged" in lines[1], r.stdout
    ln = lines[0].split()
    steps = int(ln[ln.index("steps") + 1])
    assert "converged" in ln and steps % 500 == 0 and float(ln[ln.index("residual") + 1]) < 1e-8
    d, info = mph.InputParser(files[0], overrides=["sim.max_step=400000"]).derive("f64x")
    s = mph.Simulation(d, info)
    s.initialize()
    s.advance(steps)
    rho, _ = s.update_macroscopic()
    got = np.load(tmp_path / "out" / "domain0000" / "final" / "density.npy").reshape(-1)
    assert np.array_equal(got, rho * info.ref_density)
