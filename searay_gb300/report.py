"""Wave-data files of a volume's report (modules/volume.py:626-641).

After ``track`` the reference's volume keeps the five arrays that ``track`` returned, and its
``Report`` writes each one with ``np.save`` as ``<basename>_<volume name>_<propagator>_<field>.npy``.
The fields are ``wave`` (A), ``j`` (J), ``chi`` (chiNL), ``plasma`` (ne) and ``plot_ext`` (the
(8,) extent dom4d).  ``write_wave_data`` writes the same files, with the same contents and dtypes,
from the tuple that :func:`searay_gb300.track` or :func:`searay_gb300.paraxial.track` returns, so
SeaRay's post-processing finds them where it looks.  The rest of ``Report`` (rays, orbits) is the
volume's own and is not on the propagation path.
"""
import numpy as np

FIELDS = ("wave", "j", "chi", "plasma", "plot_ext")
PROPAGATORS = {"uppe": "UPPE", "paraxial": "paraxial"}


def wave_data_paths(basename, volume_name, propagator="uppe"):
    """The five file names that ``Report`` writes for a volume (modules/volume.py:629-641)."""
    if propagator not in PROPAGATORS:
        raise ValueError(f"no wave data for propagator {propagator!r}; expected one of {sorted(PROPAGATORS)}")
    return [f"{basename}_{volume_name}_{propagator}_{field}.npy" for field in FIELDS]


def write_wave_data(basename, volume_name, outputs, propagator="uppe"):
    """Save ``outputs`` = (A, J, chiNL, ne, dom4d) under the report's names; returns the paths.

    Prints the reference's progress line (``Write UPPE wave data...``) before writing."""
    paths = wave_data_paths(basename, volume_name, propagator)
    if len(outputs) != len(FIELDS):
        raise ValueError(f"expected the {len(FIELDS)} arrays that track returns, got {len(outputs)}")
    print(f"    Write {PROPAGATORS[propagator]} wave data...")
    for path, data in zip(paths, outputs):
        with open(path, "wb") as f:
            np.save(f, np.asarray(data))
    return paths
