"""The C ABI library: loads, exports every entry point declared in
include/mph.h, and reports errors as codes (no compute without a GPU)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "mph.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mph_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(mph):
    lib = C.CDLL(mph.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(mph.EXPORTS) == names


def test_abi_version(mph):
    assert mph.lib().mph_abi_version() == 1


def test_null_arguments_are_errors(mph):
    L = mph.lib()
    assert L.mph_create(None, None) == 1
    assert L.mph_set_f(None, None) == 1
    assert L.mph_advance(None, 1) == 1
    assert b"NULL" in L.mph_last_error() or len(L.mph_last_error()) > 0


def test_create_rejects_bad_descriptions(mph):
    with pytest.raises(mph.MphError) as e:
        mph.Simulation(mph.make_desc("D2Q9", (0, 4), 1.0))
    assert e.value.code == 1
    d = mph.make_desc("D2Q9", (4, 4), 1.0)
    d.q = 19
    with pytest.raises(mph.MphError):
        mph.Simulation(d)
    d = mph.make_desc("D2Q9", (4, 4), 2.5)
    with pytest.raises(mph.MphError) as e:
        mph.Simulation(d)
    assert e.value.code == 2
    d = mph.make_desc("D2Q9", (4, 4), 1.0, faces=["Inflow", "Outflow", "PressureOutlet", "NoSlip", "Periodic", "Periodic"])
    with pytest.raises(mph.MphError) as e:
        mph.Simulation(d)
    assert e.value.code == 2


def test_no_cpu_fallback_without_a_device(mph):
    """Without a CUDA device the handle cannot be created: the product has no
    CPU path to fall back to."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(mph.MphError) as e:
        mph.Simulation(mph.make_desc("D2Q9", (8, 8), 1.0))
    assert e.value.code == 3


@pytest.mark.parametrize("name", ["f64", "f64_fast", "f32", "f16s", "bf16s", "f64x", "f16c", "f16w"])
def test_every_precision_name_is_a_known_storage(name, mph):
    """Every precision name maps to a storage the library knows: without a
    device, creating a single handle or a batch in it gets as far as the first
    CUDA call (MPH_ERR_CUDA), while an unknown precision code is rejected
    before it (MPH_ERR_ARG / MPH_ERR_UNSUPPORTED)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    d = mph.make_desc("D2Q9", (8, 8), 1.0, precision=name)
    assert d.precision == mph.PRECISION[name]
    with pytest.raises(mph.MphError) as e:
        mph.Simulation(d)
    assert e.value.code == 3
    with pytest.raises(mph.MphError) as e:
        mph.Batch([d])
    assert e.value.code == 3


def test_unknown_precision_codes_are_rejected_before_the_device(mph):
    d = mph.make_desc("D2Q9", (8, 8), 1.0)
    for code in (-1, len(mph.PRECISION), 99):
        d.precision = code
        with pytest.raises(mph.MphError) as e:
            mph.Simulation(d)
        assert e.value.code == 1
        with pytest.raises(mph.MphError) as e:
            mph.Batch([d])
        assert e.value.code == 4
