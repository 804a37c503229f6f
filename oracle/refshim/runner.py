"""Test infrastructure only (oracle): run the reference's own UPPE path on host cores.

``reference_track(vol_dict)`` calls the reference's unmodified ``uppe_kernel.track``
(``modules/uppe_kernel.py:333-424``) with its own OpenCL kernels, compiled as C++ by the
``pyopencl`` stand-in in this folder.  It needs the reference source tree: the folder named by ``SEARAY_REF``, by ``set_reference()``,
or else the one that the build recipe recorded in ``oracle/_ref/reference_root.txt`` when it
compiled the reference's kernels there.  It runs only where that tree exists; it is used to generate
the golden fixtures under ``tests/golden/`` and never at test or bench time on a GPU machine.
"""
import contextlib
import io
import os
import pathlib
import sys

import numpy as np

_HERE = pathlib.Path(__file__).resolve().parent
RECORD = _HERE.parent / "_ref" / "reference_root.txt"


def _resolve():
    if os.environ.get("SEARAY_REF"):
        return pathlib.Path(os.environ["SEARAY_REF"])
    if RECORD.exists():
        return pathlib.Path(RECORD.read_text().strip())
    return None


REF = _resolve()


def set_reference(path):
    """Use the reference source tree at ``path`` (before the first reference call)."""
    global REF
    REF = pathlib.Path(path)


def record_reference(path):
    """Remember ``path`` as the reference tree for later processes (written by the build recipe)."""
    set_reference(path)
    RECORD.parent.mkdir(exist_ok=True)
    RECORD.write_text(str(REF) + "\n")


def available():
    return REF is not None and (REF / "modules" / "uppe_kernel.py").exists()


def _setup_path():
    for p in (str(REF / "modules"), str(REF), str(_HERE)):
        if p in sys.path:
            sys.path.remove(p)
    # the stand-in pyopencl must shadow any other, and the reference modules import each other
    # both as top-level modules and as ``modules.x``
    sys.path.insert(0, str(REF))
    sys.path.insert(0, str(REF / "modules"))
    sys.path.insert(0, str(_HERE))


_CL = None


def cl_refs():
    """The reference's own ``init.cl_refs`` with its programs built through the stand-in."""
    global _CL
    if _CL is None:
        _setup_path()
        import pyopencl
        import init
        ctx = pyopencl.Context()
        q = pyopencl.CommandQueue(ctx)
        cl = init.cl_refs(ctx, ctx.devices[0], q)
        for prog in ("fft", "uppe", "paraxial", "ionization", "rotations"):
            cl.add_program(str(REF / "kernels"), prog)
        _CL = cl
    return _CL


def modules():
    """Import and return the reference modules used to build UPPE inputs."""
    _setup_path()
    import importlib
    names = ("uppe_kernel", "grid_tools", "caustic_tools", "ionization", "photoionization_base",
             "dispersion", "input_tools", "volume", "rotations", "paraxial_kernel")
    return {n: importlib.import_module(n) for n in names}


class DensityObject:
    """Minimal volume object: ``GetRelDensity`` as ``AnalyticDensity`` computes it
    (``modules/volume.py:669-674``), from the dict's ``density lambda``."""

    def __init__(self, vol_dict):
        self.vol_dict = vol_dict

    def GetRelDensity(self, xp):
        x = xp[..., 1]
        y = xp[..., 2]
        z = xp[..., 3]
        r2 = np.einsum("...i,...i", xp[..., 1:3], xp[..., 1:3])
        return self.vol_dict["density lambda"](x, y, z, r2)


def reference_track(vol_dict, quiet=True):
    """Run ``uppe_kernel.track`` with no rays entering the grid (the ``incoming wave`` route)."""
    cl = cl_refs()
    m = modules()
    vd = dict(vol_dict)
    if "object" not in vd:
        vd["object"] = DensityObject(vd)
    # two bundles of 4 rays near the axis at the carrier frequency; the final ray relaunch
    # (caustic_tools.py RelaunchRays) only moves these rays and does not touch the wave data
    xp = np.zeros((2, 4, 8))
    xp[..., 4] = 1.0
    xp[..., 7] = 1.0
    ang = np.arange(8).reshape(2, 4) * 0.4
    xp[..., 1] = 1e-3 * np.cos(ang)
    xp[..., 2] = 1e-3 * np.sin(ang)
    eikonal = np.zeros((2, 4))
    vg = np.zeros((2, 4, 4))
    out = io.StringIO()
    with contextlib.redirect_stdout(out) if quiet else contextlib.nullcontext():
        A, J, chi, ne, dom4d = m["uppe_kernel"].track(cl, xp, eikonal, vg, vd)
    return A, J, chi, ne, dom4d, out.getvalue()


def reference_track_rays(vol_dict, xp, eikonal, vg, quiet=True):
    """Run ``uppe_kernel.track`` on the given rays (no ``incoming wave``: the wave starts from
    ``GetBoundaryFields``); returns its outputs and the relaunched ray arrays (copies)."""
    cl = cl_refs()
    m = modules()
    vd = dict(vol_dict)
    if "object" not in vd:
        vd["object"] = DensityObject(vd)
    xp, eikonal, vg = np.array(xp), np.array(eikonal), np.array(vg)
    out = io.StringIO()
    with contextlib.redirect_stdout(out) if quiet else contextlib.nullcontext():
        A, J, chi, ne, dom4d = m["uppe_kernel"].track(cl, xp, eikonal, vg, vd)
    return A, J, chi, ne, dom4d, xp, eikonal, vg


def reference_paraxial(vol_dict, quiet=True):
    """Run ``paraxial_kernel.track`` (``modules/paraxial_kernel.py:367-443``) with no rays entering
    the grid (the ``incoming wave`` route), with the same harmless ray bundles as reference_track."""
    cl_refs()
    m = modules()
    vd = dict(vol_dict)
    if "object" not in vd:
        vd["object"] = DensityObject(vd)
    xp = np.zeros((2, 4, 8))
    xp[..., 4] = 1.0
    xp[..., 7] = 1.0
    ang = np.arange(8).reshape(2, 4) * 0.4
    xp[..., 1] = 1e-3 * np.cos(ang)
    xp[..., 2] = 1e-3 * np.sin(ang)
    eikonal = np.zeros((2, 4))
    vg = np.zeros((2, 4, 4))
    out = io.StringIO()
    with contextlib.redirect_stdout(out) if quiet else contextlib.nullcontext():
        A, J, chi, ne, dom4d = m["paraxial_kernel"].track(_CL, xp, eikonal, vg, vd)
    return A, J, chi, ne, dom4d, out.getvalue()


def reference_paraxial_rays(vol_dict, xp, eikonal, vg, quiet=True):
    """Run ``paraxial_kernel.track`` on the given rays (no ``incoming wave``); returns its outputs and
    the relaunched ray arrays (copies)."""
    cl_refs()
    m = modules()
    vd = dict(vol_dict)
    if "object" not in vd:
        vd["object"] = DensityObject(vd)
    xp, eikonal, vg = np.array(xp), np.array(eikonal), np.array(vg)
    out = io.StringIO()
    with contextlib.redirect_stdout(out) if quiet else contextlib.nullcontext():
        A, J, chi, ne, dom4d = m["paraxial_kernel"].track(_CL, xp, eikonal, vg, vd)
    return A, J, chi, ne, dom4d, xp, eikonal, vg
