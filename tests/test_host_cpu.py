"""Host-side set-up of the GB300 propagator against the oracle and the reference's fixtures and
known answers (no GPU)."""
import numpy as np
import pytest

import replay
from oracle import uppe_oracle as O
from searay_gb300 import dispersion, grid, ionization, uppe


@pytest.mark.parametrize("name", replay.CASE_NAMES)
def test_grid_matches_oracle(name):
    vd, _ = replay.load_case(name)
    g = grid.VolumeGrid(vd)
    go = O.Grid(vd)
    for attr in ("w", "x1", "x2", "kr2", "plot_ext"):
        np.testing.assert_array_equal(getattr(g, attr), getattr(go, attr))
    assert g.dt == go.dt and g.dw == go.dw
    if not g.cartesian:
        np.testing.assert_array_equal(g.H, go.H)
        np.testing.assert_array_equal(g.Lambda, go.Lambda)


def test_hankel_basis_matches_reference():
    d = np.load(replay.HERE / "hankel_bases.npz")
    for (Nr, dr, mmax, Nk) in ((32, 25.0, 0, 24), (16, 37.5, 2, 12)):
        key = f"Nr{Nr}_mmax{mmax}_Nk{Nk}"
        H, vals, lam = grid.hankel_eigenbasis(Nr, dr, mmax, Nk)
        np.testing.assert_allclose(H, d[key + "_H"], rtol=0, atol=1e-13)
        np.testing.assert_allclose(vals, d[key + "_vals"], rtol=1e-13)
        # orthogonality H H^T = I for a full basis
        Hf, _, _ = grid.hankel_eigenbasis(Nr, dr, mmax, Nr)
        for m in range(Hf.shape[2]):
            np.testing.assert_allclose(Hf[:, :, m] @ Hf[:, :, m].T, np.eye(Nr), atol=1e-12)


@pytest.mark.parametrize("name", ["cart_ion", "cyl_az_adk", "cart_series"])
def test_rate_coefficients_match_reference(name):
    vd, exp = replay.load_case(name)
    rc = ionization.RateCoefficients(vd["ionizer"])
    ro = O.RateCoefficients(vd["ionizer"])
    assert (rc.C1, rc.C2, rc.C3) == (ro.C1, ro.C2, ro.C3)
    assert rc.field_conv == ro.field_conv and rc.rate_conv == ro.rate_conv
    if not rc.explicit:
        np.testing.assert_allclose(rc.clog, exp["rate"]["clog_reference"], rtol=1e-9)


def test_simple_air_matches_reference_chi():
    d = np.load(replay.HERE / "uppe_cart_ion.npz")
    air = dispersion.SimpleAir(0.8e-6 / (2 * np.pi))
    np.testing.assert_allclose(air.chi(d["w_nodes"]), d["chi_w"].real, rtol=1e-14, atol=0)


def test_ionization_known_answers():
    """The rate known answers of the reference's test/ionization_test.py:6-15."""
    h = ionization.HydrogenAU(False, 0.5, 1.0, 0, 0, 0, 0)
    assert h.Rate(0.1 - h.cutoff_field) == pytest.approx(0.0509, 1e-3)
    au = ionization.AtomicUnits()
    adk = ionization.ADKAU(True, au.energy_to_au(24.58741), 1.0)
    assert adk.Rate(0.1 - adk.cutoff_field) == pytest.approx(4.546e-7, 1e-2)


def test_rate_models_match_reference_classes():
    from oracle.refshim import runner
    if not runner.available():
        pytest.skip("reference tree not present")
    m = runner.modules()
    x1 = 0.8e-6 / (2 * np.pi)
    helper = m["input_tools"].InputHelper(x1)
    U = helper.dnum("12.07 eV")
    for mine, theirs in ((ionization.PPT_Tunneling(x1, False, U, 0.53), m["ionization"].PPT_Tunneling(x1, False, U, 0.53)),
                         (ionization.ADK(x1, False, U, 1.0), m["ionization"].ADK(x1, False, U, 1.0))):
        np.testing.assert_allclose(mine.GetCoeff(), theirs.GetCoeff(), rtol=1e-13)
    air_ref = m["dispersion"].SimpleAir(x1)
    w = np.linspace(0.1, 2.5, 50)
    np.testing.assert_allclose(dispersion.SimpleAir(x1).GroupVelocityMagnitude(w), air_ref.GroupVelocityMagnitude(w), rtol=1e-13)


def test_track_rejects_bad_grids_before_device_use():
    vd, _ = replay.load_case("cart_ion")
    for N, msg in (((128, 16, 16, 2), "w-nodes"), ((129, 12, 16, 2), "x-nodes"), ((129, 16, 24, 2), "y-nodes")):
        v = dict(vd)
        v["wave grid"] = N
        with pytest.raises(ValueError, match=msg):
            uppe.track(None, None, None, None, v)


def test_rotator_matches_reference():
    """Rotator tables (rotations.py:15-44) against those of the reference's own Rotator stored with
    the N2 Raman case, and the normalisation sum (2j+1) rho0_j = 1 of the thermal populations."""
    import cases
    from searay_gb300 import rotations
    vd, _ = replay.load_case("cyl_raman")
    rot = rotations.Rotator(*cases.rotator_args(cases.CASES["cyl_raman"]["rotator"]))
    ref = vd["rotator"]
    np.testing.assert_allclose(rot.Wj, ref.Wj, rtol=1e-15, atol=0)
    np.testing.assert_allclose(rot.Tj, ref.Tj, rtol=1e-15, atol=0)
    assert rot.dalpha == ref.dalpha and rot.hbar == ref.hbar
    j = np.arange(rot.wj.shape[0])
    assert np.sum((2 * j + 1) * rot.rho0jm) == pytest.approx(1.0, rel=1e-14)
    assert rot.Wj[0] == 0 and rot.Wj[1] == 0 and rot.Tj[0] == 0 and rot.Tj[1] == 0


@pytest.mark.parametrize("name", replay.PARAXIAL_CASE_NAMES)
def test_paraxial_material_tables_match_oracle(name):
    """The envelope tables that paraxial.Material hands to the device (f(w), k0(w), the gas density;
    paraxial_kernel.py:67-91) equal the oracle's, in FFT order."""
    from oracle import paraxial_oracle as PO
    from searay_gb300 import paraxial

    class FakeDevice:
        def set_material(self, fw, k0, ng):
            self.tables = (fw, k0, ng)
            return True

    vd, _ = replay.load_case(name)
    orc = PO.ParaxialOracle(vd)
    g = grid.VolumeGrid(vd)
    dev = FakeDevice()
    chi = vd["dispersion inside"].chi(g.w).astype(np.cdouble)
    mat = paraxial.Material(dev, g, vd["wave coordinates"], None, chi, vd.get("chi3", 0.0), vd["density reference"],
                            orc.w0, orc.ngrp, orc.n0, vd["density lambda"])
    for z in (-3000.0, 0.0, 2500.0):
        mat.UpdateMaterial(z)
        orc.mat.update(z)
        fw, k0, ng = dev.tables
        np.testing.assert_array_equal(fw, orc.mat.fw)
        np.testing.assert_array_equal(k0, orc.mat.k0)
        np.testing.assert_array_equal(ng, orc.mat.ng)


def test_paraxial_grid_checks():
    """The ValueErrors of paraxial_kernel.py:393-398, raised before any device work."""
    from searay_gb300 import paraxial
    vd, _ = replay.load_case("par_cart_ion")
    for N, msg in (((129, 16, 16, 2), "w-nodes"), ((128, 12, 16, 2), "x-nodes"), ((128, 16, 24, 2), "y-nodes")):
        v = dict(vd)
        v["wave grid"] = N
        with pytest.raises(ValueError, match=msg):
            paraxial.track(None, None, None, None, v)


def test_bench_byte_model_counts_zero_current_slices():
    """bench.py's algorithmic bytes of the Cartesian fused evaluation tail: 44 B per point on the
    slices with current (40 / 48 / 48 / 40 over the RK stages), 32 / 0 / 24 / 0 on the slices at and
    above the nonlinear cut, whose stages 2 and 4 have nothing to do (65 of 513 slices on the
    filament grid: 40.2 B per point); the full 44 B when the nonlinear band reaches the top of the
    frequency band; and the cut index the library computes (int(nl_hi / dw) of the grid)."""
    import sys
    import pathlib
    sys.path.insert(0, str(pathlib.Path(__file__).resolve().parents[1]))
    import bench
    from searay_gb300 import workloads
    vd = workloads.cart_filament_128()
    g = grid.VolumeGrid(vd)
    jhi = int(vd["nonlinear band"][1] / g.dw)
    assert jhi == 448
    f = (513 - jhi) / 513
    assert bench.cart_forward_bytes(vd) == pytest.approx((1 - f) * 44 + f * 14)
    assert bench.cart_forward_bytes(vd) == pytest.approx(40.2, abs=0.05)
    full = dict(vd)
    full["nonlinear band"] = vd["frequency band"]
    assert bench.cart_forward_bytes(full) == pytest.approx(44.0)
    m = bench.class_models(vd)
    assert m["time_pass"]["bytes"] == 16 * 513 * 128 * 128


@pytest.mark.parametrize("propagator,case", [("uppe", "cart_ion"), ("paraxial", replay.PARAXIAL_CASE_NAMES[0])])
def test_report_writes_reference_wave_files(tmp_path, capsys, propagator, case):
    """The wave-data files of a volume's report: names, contents and dtypes as modules/volume.py:626-641
    writes them from track's five returns."""
    from searay_gb300 import report
    _, exp = replay.load_case(case)
    outputs = tuple(exp[k] for k in ("A", "J", "chi", "ne", "dom4d"))
    base = str(tmp_path / "run")
    paths = report.write_wave_data(base, "vol0", outputs, propagator)
    label = "UPPE" if propagator == "uppe" else "paraxial"
    assert f"Write {label} wave data..." in capsys.readouterr().out
    assert [p.rsplit("/", 1)[1] for p in paths] == [
        f"run_vol0_{propagator}_{f}.npy" for f in ("wave", "j", "chi", "plasma", "plot_ext")]
    for p, a in zip(paths, outputs):
        b = np.load(p)
        assert b.dtype == a.dtype and b.shape == a.shape
        np.testing.assert_array_equal(b, a)
    with pytest.raises(ValueError):
        report.wave_data_paths(base, "vol0", "eikonal")
    with pytest.raises(ValueError):
        report.write_wave_data(base, "vol0", outputs[:4], propagator)


def test_product_code_never_reaches_the_oracle():
    """The package (Python host, CUDA sources, C header) imports, loads or names neither the oracle
    nor scratch files: the oracle is test infrastructure and the product has no CPU fallback."""
    import pathlib
    import re
    root = pathlib.Path(__file__).resolve().parent.parent
    files = [p for p in (root / "searay_gb300").rglob("*") if p.suffix in (".py", ".cu", ".cuh", ".h")]
    files += list((root / "include").glob("*.h"))
    assert len(files) > 10
    pat = re.compile(r"\boracle\b|\b_work\b|refshim")
    hits = [f"{p.relative_to(root)}:{i + 1}" for p in files
            for i, line in enumerate(p.read_text().splitlines()) if pat.search(line)]
    assert hits == []


def test_programmatic_launches_wait_for_their_predecessor():
    """Every kernel launched with the programmatic-dependent-launch attribute (launch_pdl) must call
    pdl_begin() before touching global memory: without its griddepcontrol.wait it could read the
    previous kernel's output before that kernel has finished.  Source check over csrc/: each such
    kernel's body calls pdl_begin() ahead of its first loop, branch or asynchronous copy."""
    import pathlib
    import re
    csrc = pathlib.Path(__file__).resolve().parent.parent / "searay_gb300" / "csrc"
    sources = {p: p.read_text() for p in list(csrc.glob("*.cu")) + list(csrc.glob("*.cuh"))}
    launched = set()
    for text in sources.values():
        launched.update(re.findall(r"launch_pdl\((k_\w+)", text))
    assert launched, "no programmatic launches found"
    for name in sorted(launched):
        bodies = []
        for text in sources.values():
            for m in re.finditer(r"__global__[^;{]*?\b" + name + r"\s*\(", text):
                depth, j = 0, m.end() - 1
                while True:
                    if text[j] == "(":
                        depth += 1
                    elif text[j] == ")":
                        depth -= 1
                        if depth == 0:
                            break
                    j += 1
                k = text.index("{", j)
                if ";" in text[j + 1:k]:
                    continue  # a declaration
                bodies.append(text[k + 1:])
        assert bodies, name
        for body in bodies:
            head = body[:body.index("pdl_begin();")] if "pdl_begin();" in body else None
            assert head is not None, f"{name} is launched with launch_pdl but never calls pdl_begin()"
            # nothing before pdl_begin reads or writes global memory: no loops, no cp.async, no
            # indexing of kernel arguments (declarations and shared-memory set-up only)
            assert not re.search(r"\bfor\s*\(|cp_async|\bif\s*\(", head), (name, head[-300:])
