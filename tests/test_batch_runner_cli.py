"""Argument handling of the host drivers (mph_batch_run, mph_run) that needs
no GPU: usage, an unknown precision, missing inputs files."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
INPUTS = os.path.join(HERE, "inputs", "cavity2d.inputs")


def test_usage_and_precision_errors(mph, tmp_path):
    exe = os.path.join(os.path.dirname(mph.__file__), "_build", "mph_batch_run")
    assert os.access(exe, os.X_OK)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([exe, INPUTS, "mph.precision=f128"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 1 and "mph.precision" in r.stderr
    r = subprocess.run([exe, str(tmp_path / "missing.inputs")], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 1 and r.stderr.startswith("mph_batch_run:")


def test_single_driver_usage_and_precision_errors(mph, tmp_path):
    """mph_run: usage without arguments, a bad precision and a missing inputs
    file are reported before any device work."""
    exe = os.path.join(os.path.dirname(mph.__file__), "_build", "mph_run")
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([exe, INPUTS, "mph.precision=f128"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 1 and "mph.precision" in r.stderr and r.stderr.startswith("mph_run:")
    r = subprocess.run([exe, str(tmp_path / "missing.inputs")], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 1 and r.stderr.startswith("mph_run:")
