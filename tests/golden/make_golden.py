"""Generate the golden fixtures in this folder from the reference itself.

Runs SeaRay's own unmodified UPPE path (``modules/uppe_kernel.py:333-424`` with its OpenCL kernels
``kernels/{fft,uppe,ionization,paraxial,rotations}.cl`` compiled as C++ by ``oracle/refshim``) on
the cases of ``cases.py``, and its paraxial path (``modules/paraxial_kernel.py:367-443``) on the
paraxial cases, and stores, per case, the resolved inputs (incoming field, chi(w), rate
coefficients) and the outputs (A, J, chiNL, ne on every diagnostic plane after the first, dom4d).
Also stores reference Hankel bases (``grid_tools.HankelTransformTool``).

Needs the reference source tree, given by ``--reference PATH`` (or ``SEARAY_REF``)::

    python tests/golden/make_golden.py --reference PATH [case ...]

With case names, only those fixtures are written (and not the Hankel bases).
"""
import json
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE))

from oracle.refshim import runner  # noqa: E402
import cases  # noqa: E402


def build_ref_case(name, m):
    c = cases.CASES[name] if name in cases.CASES else cases.PARAXIAL_CASES[name]
    keys = dict(c["keys"])
    helper = m["input_tools"].InputHelper(cases.MKS_LENGTH)
    disp = m["dispersion"]
    if c["medium"] == "SimpleAir":
        medium = disp.SimpleAir(cases.MKS_LENGTH)
    elif c["medium"] == "Vacuum":
        medium = disp.Vacuum()
    else:
        raise ValueError(c["medium"])
    if keys.get("window speed") == "vg":
        keys["window speed"] = float(medium.GroupVelocityMagnitude(1.0))
    iz = None
    if c["ionizer"] is not None:
        spec = c["ionizer"]
        Uion = helper.dnum(f"{spec['Uion_eV']} eV")
        cls = getattr(m["ionization"], spec["kind"])
        if spec["kind"] in ("PPT", "PMPB", "StitchedPPT"):
            iz = cls(cases.MKS_LENGTH, False, Uion, spec["Z"], lstar=0, l=0, m=0, w0=1.0, terms=spec.get("terms", 40))
        else:
            iz = cls(cases.MKS_LENGTH, False, Uion, spec["Z"])
    vd = dict(keys)
    vd["dispersion inside"] = medium
    vd["ionizer"] = iz
    if c.get("rotator") is not None:
        vd["rotator"] = m["rotations"].Rotator(*cases.rotator_args(c["rotator"]))
    vd["density lambda"] = cases.density_lambda(c["density"])
    vd["incoming wave"] = cases.make_wave(c["wave"], keys["size"][0])
    return vd, medium, iz


def main(names=None):
    if not runner.available():
        raise SystemExit("reference tree not found")
    m = runner.modules()
    for name in names or (list(cases.CASES) + list(cases.PARAXIAL_CASES)):
        vd, medium, iz = build_ref_case(name, m)
        paraxial = name in cases.PARAXIAL_CASES
        if paraxial:
            A, J, chi, ne, dom4d, log = runner.reference_paraxial(vd)
        else:
            A, J, chi, ne, dom4d, log = runner.reference_track(vd)
        N = vd["wave grid"]
        w = A.shape[0]
        # resolved inputs, so the case can be replayed without the reference classes
        band = vd["frequency band"]
        w_nodes = 0.5 * (band[0] + band[1]) + np.linspace(-(band[1] - band[0]) / 2, (band[1] - band[0]) / 2 - (band[1] - band[0]) / N[0], N[0])
        rate = {}
        if iz is not None:
            izr = m["ionization"].Ionizer(iz)
            rate = {"mks_length": iz.get_mks_length(), "coeff": list(iz.GetCoeff())}
            if izr.C1 == 0.0:
                E_table = np.logspace(np.log10(izr.cutoff_field * 2), np.log10(1), 256)
                rate["E_table"] = E_table.tolist()
                rate["rate_table"] = iz.Rate(E_table).tolist()
                rate["clog_reference"] = [float(v) for v in izr.Clog]
        meta = {k: v for k, v in vd.items() if isinstance(v, (int, float, str, tuple, list)) and k not in ("incoming wave",)}
        meta["density"] = (cases.PARAXIAL_CASES if paraxial else cases.CASES)[name]["density"]
        meta["propagator"] = "paraxial" if paraxial else "uppe"
        meta["rate"] = rate
        meta["evals_log"] = log.strip().splitlines()[-1] if log.strip() else ""
        rot = vd.get("rotator")
        meta["rotator"] = {} if rot is None else {
            "Wj": [[float(v.real), float(v.imag)] for v in rot.Wj], "Tj": [float(v) for v in rot.Tj],
            "dalpha": float(rot.dalpha), "hbar": float(rot.hbar)}
        np.savez_compressed(
            HERE / (f"{name}.npz" if paraxial else f"uppe_{name}.npz"),
            meta=np.array(json.dumps(meta)),
            w_nodes=w_nodes,
            chi_w=np.asarray(medium.chi(w_nodes)).astype(np.cdouble),
            A0=A[..., 0],
            A=A[..., 1:], J=J[..., 1:], chi=chi[..., 1:], ne=ne[..., 1:], dom4d=dom4d)
        print(name, A.shape, "max|A|", np.abs(A[..., -1]).max(), "max|ne|", np.abs(ne).max(), meta["evals_log"], file=sys.stderr)
        assert w == N[0]
    if names:
        return
    # Hankel bases from the reference's HankelTransformTool (grid_tools.py:252-298)
    gt = m["grid_tools"]
    bases = {}
    for (Nr, dr, mmax, Nk) in ((32, 25.0, 0, 24), (16, 37.5, 2, 12)):
        T = gt.HankelTransformTool(Nr, dr, mmax, None, Nk)
        key = f"Nr{Nr}_mmax{mmax}_Nk{Nk}"
        bases[key + "_H"] = T.H
        bases[key + "_vals"] = T.vals
        bases[key + "_Lambda"] = T.Lambda
    np.savez_compressed(HERE / "hankel_bases.npz", **bases)


def _args(argv):
    """Strip ``--reference PATH`` from the arguments and point the reference runner at PATH."""
    argv = list(argv)
    if "--reference" in argv:
        i = argv.index("--reference")
        runner.set_reference(argv[i + 1])
        del argv[i:i + 2]
    return argv


if __name__ == "__main__":
    main(_args(sys.argv[1:]))
