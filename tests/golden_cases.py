"""Loader of the committed golden fixtures (tests/golden/)."""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

_cache = {}


def cases():
    if "cases" not in _cache:
        z = np.load(os.path.join(GOLDEN, "cases.npz"))
        _cache["arrays"] = {k: z[k] for k in z.files}
        _cache["cases"] = json.loads(str(_cache["arrays"]["index"]))
    return _cache["cases"]


def arr(name, key):
    cases()
    return _cache["arrays"][f"{name}/{key}"]


def units():
    with open(os.path.join(GOLDEN, "units.json")) as fh:
        return json.load(fh)


def oracle_config(case, O):
    return O.Config(case["lattice"], tuple(case["n"]), omega=float.fromhex(case["omega"]), faces=case["faces"],
                    face_rho=[float.fromhex(x) for x in case["face_rho"]],
                    face_U=[[float.fromhex(x) for x in U] for U in case["face_U"]],
                    force=tuple(float.fromhex(x) for x in case["force"]) if case["force"] else None)


def product_desc(case, m, precision="f64"):
    return m.make_desc(case["lattice"], tuple(case["n"]), float.fromhex(case["omega"]), faces=case["faces"],
                       face_rho=[float.fromhex(x) for x in case["face_rho"]],
                       face_U=[[float.fromhex(x) for x in U] for U in case["face_U"]],
                       force=tuple(float.fromhex(x) for x in case["force"]) if case["force"] else None,
                       precision=precision)
