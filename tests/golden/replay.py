"""Rebuild a stored parity case as a SeaRay volume input dictionary, without the reference tree.

The fixture ``uppe_<case>.npz`` (written by ``make_golden.py``) holds the resolved inputs: the
incoming field on the grid, chi(w) of the medium, the rate-model coefficients and (series form) the
rate table the fit is made from.  The small duck-typed objects below stand in for the reference's
dispersion and rate-model classes and expose just the methods ``uppe_kernel.track`` and
``ionization.Ionizer`` call: ``chi(w)``, ``GetCoeff()``, ``get_mks_length()``, ``Rate(E)``, and the
rotator's transition table (``Wj``, ``Tj``, ``dalpha``, ``hbar``).
"""
import json
import pathlib

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
CASE_NAMES = ("cyl_kerr", "cart_ion", "cyl_az_adk", "cart_series", "cyl_raman")
PARAXIAL_CASE_NAMES = ("par_cart_ion", "par_cyl_raman", "par_cyl_az_adk")


class StoredDispersion:
    def __init__(self, w_nodes, chi_w):
        self.w_nodes = w_nodes
        self.chi_w = chi_w

    def chi(self, w):
        w = np.asarray(w)
        if w.shape == self.w_nodes.shape and np.allclose(w, self.w_nodes, rtol=0, atol=1e-12):
            return self.chi_w.copy()
        raise ValueError("stored dispersion queried off its frequency nodes")


class StoredRate:
    def __init__(self, rate):
        self.mks_length = rate["mks_length"]
        self.coeff = tuple(rate["coeff"])
        self.E_table = np.array(rate.get("E_table", []))
        self.rate_table = np.array(rate.get("rate_table", []))

    def get_mks_length(self):
        return self.mks_length

    def GetCoeff(self):
        return self.coeff

    def Rate(self, E):
        E = np.asarray(E)
        if E.shape == self.E_table.shape and np.allclose(E, self.E_table, rtol=1e-14, atol=0):
            return self.rate_table.copy()
        raise ValueError("stored rate queried off its table")


class StoredRotator:
    """The attributes of the reference's rotations.Rotator that AddChi reads (Wj, Tj, dalpha, hbar)."""

    def __init__(self, rot):
        self.Wj = np.array([complex(a, b) for a, b in rot["Wj"]])
        self.Tj = np.array(rot["Tj"], dtype=float)
        self.dalpha = rot["dalpha"]
        self.hbar = rot["hbar"]


def density_lambda(expr):
    code = compile(expr, "<density>", "eval")
    return lambda x, y, z, r2: eval(code, {"np": np}, {"x": x, "y": y, "z": z, "r2": r2})


def load_case(name):
    """Return (vol_dict, expected) for a stored case; expected holds A, J, chi, ne (planes >= 1)
    and dom4d as the reference produced them."""
    d = np.load(HERE / (f"{name}.npz" if name in PARAXIAL_CASE_NAMES else f"uppe_{name}.npz"))
    meta = json.loads(str(d["meta"]))
    vd = {}
    for k, v in meta.items():
        if k in ("density", "rate", "evals_log", "rotator", "propagator"):
            continue
        vd[k] = tuple(v) if isinstance(v, list) else v
    A0 = d["A0"]
    vd["incoming wave"] = lambda w, x1, x2, _a=A0: _a.copy()
    vd["dispersion inside"] = StoredDispersion(d["w_nodes"], d["chi_w"])
    vd["ionizer"] = StoredRate(meta["rate"]) if meta["rate"] else None
    vd["density lambda"] = density_lambda(meta["density"])
    if meta.get("rotator"):
        vd["rotator"] = StoredRotator(meta["rotator"])
    expected = {k: d[k] for k in ("A", "J", "chi", "ne", "dom4d")}
    expected["evals_log"] = meta.get("evals_log", "")
    expected["rate"] = meta["rate"]
    return vd, expected
