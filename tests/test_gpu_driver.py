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
