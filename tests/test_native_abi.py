"""The C-ABI library: it builds, loads, exports every entry point include/searay_uppe.h declares,
and the ctypes mirror of UppeConfig has the C layout.  No device calls (runs without a GPU)."""
import ctypes
import pathlib
import re
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "searay_uppe.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(uppe_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def built():
    from searay_gb300 import build
    build.build()
    from searay_gb300 import _native
    return _native.lib()


def test_exports_every_declared_symbol(built):
    from searay_gb300 import _native
    names = declared_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(built, n), n
    assert set(names) == set(_native.EXPORTS)


def test_config_struct_layout(tmp_path):
    from searay_gb300 import _native
    src = tmp_path / "probe.c"
    fields = [f[0] for f in _native.UppeConfig._fields_]
    body = "\n".join(f'printf("%zu ", offsetof(UppeConfig, {f}));' for f in fields)
    src.write_text(f'#include <stdio.h>\n#include <stddef.h>\n#include "searay_uppe.h"\n'
                   f'int main(void){{ {body} printf("%zu\\n", sizeof(UppeConfig)); return 0; }}\n')
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), "-o", str(exe), str(src)], check=True)
    out = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    offs = [getattr(_native.UppeConfig, f).offset for f in fields] + [ctypes.sizeof(_native.UppeConfig)]
    assert out == offs


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    from searay_gb300 import _native
    monkeypatch.setattr(_native, "_LIB", None)
    monkeypatch.setattr(_native, "LIB_PATH", tmp_path / "absent.so")
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _native.lib()


def _config(**kw):
    """A valid Cartesian UppeConfig (17 frequencies, 16 x 1 slice) with fields overridden by kw."""
    from searay_gb300 import _native
    c = _native.UppeConfig()
    c.n0, c.n1, c.n2 = 17, 16, 1
    c.radial_modes, c.cylindrical, c.precision, c.dt = 16, 0, _native.PREC_MIXED, 0.1
    c.nl_cut_on, c.nl_cut_off, c.rate_form = 0, 17, _native.RATE_NONE
    for k, v in kw.items():
        setattr(c, k, v)
    return c


@pytest.mark.parametrize("fields,message", [
    (dict(n0=16), "2**n+1 w-nodes"),
    (dict(n0=9), "2**n+1 w-nodes"),
    (dict(n1=24), "2**n x-nodes and y-nodes"),
    (dict(n2=3), "2**n x-nodes and y-nodes"),
    (dict(n0=8193), "exceeds the 8192"),
    (dict(n1=8), "outside the supported"),
    (dict(n1=512, n2=512), "outside the supported"),
    (dict(cylindrical=1, radial_modes=17), "radial modes 17"),
    (dict(cylindrical=1, radial_modes=0), "radial modes 0"),
    (dict(precision=7), "unknown precision form 7"),
    (dict(rate_form=5), "unknown rate form 5"),
    (dict(envelope=1, n0=17), "Paraxial propagator requires 2**n w-nodes"),
    (dict(envelope=1, n0=16, n1=256, n2=256), "paraxial Cartesian slice"),
])
def test_create_rejects_bad_config_before_device_use(built, fields, message):
    """uppe_create checks the whole configuration on the host, before any CUDA call, with the
    reference's ValueError wording for the grid (modules/uppe_kernel.py:354-360)."""
    from searay_gb300 import _native
    h = ctypes.c_void_p(123)
    rc = built.uppe_create(ctypes.byref(_config(**fields)), ctypes.byref(h))
    assert rc == _native.UPPE_E_ARG
    assert h.value is None
    assert message in built.uppe_last_error(None).decode()


def test_null_arguments_return_arg_errors(built):
    """Every entry point answers a NULL handle or pointer with UPPE_E_ARG (never a crash);
    uppe_destroy(NULL) is a no-op."""
    from searay_gb300 import _native
    E = _native.UPPE_E_ARG
    n = ctypes.c_longlong()
    i = ctypes.c_int()
    assert built.uppe_create(None, None) == E
    assert b"null argument" in built.uppe_last_error(None)
    assert built.uppe_destroy(None) == _native.UPPE_OK
    assert built.uppe_set_stream(None, None) == E
    assert built.uppe_set_grid(None, None, None, None, None) == E
    assert built.uppe_set_material(None, None, None, None) == E
    assert built.uppe_load_field(None, None) == E
    assert built.uppe_rk4_step(None, 0.0, 1.0, 0.0, 0.0, None) == E
    assert built.uppe_finish(None, 0.0, None, None, None, None) == E
    assert built.uppe_eval_rhs(None, None, 0.0, None) == E
    assert built.uppe_get_field(None, None) == E
    assert built.uppe_check_finite(None, ctypes.byref(i)) == E
    assert built.uppe_set_chi3(None, 1.0) == E
    assert built.uppe_set_rotator(None, 0, None, None, 0.0, 1.0) == E
    assert built.uppe_set_field(None, None) == E
    assert built.uppe_adjoint_rk4_step(None, None, None, None, 0.0, 0.1, None) == E
    assert built.uppe_rk4_step_keep(None, 0.0, 0.1) == E
    assert built.uppe_adjoint_rk4_step_kept(None, None, None, None) == E
    assert built.uppe_adjoint_load(None, None, None) == E
    assert built.uppe_adjoint_finish(None, 0.0, None, None) == E
    assert built.uppe_profile_enable(None, 1) == E
    assert built.uppe_profile_read(None, None, None) == E
    assert built.uppe_launch_count(None, ctypes.byref(n)) == E
    assert built.uppe_step_size_noalloc(None, None, 1, 1.0, 0.4, 1e-2, None, None) == E
    assert built.uppe_class_name(2) == b"time_pass"
    assert built.uppe_class_name(99) == b"unknown"


def test_create_without_a_device_fails_loudly(built):
    """A valid configuration on a machine without a usable GPU gets UPPE_E_CUDA and the CUDA
    runtime's reason, not a handle and not a CPU fallback."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from searay_gb300 import _native
    h = ctypes.c_void_p()
    rc = built.uppe_create(ctypes.byref(_config()), ctypes.byref(h))
    assert rc == _native.UPPE_E_CUDA
    assert h.value is None
    assert built.uppe_last_error(None).decode().startswith("device allocation failed")
